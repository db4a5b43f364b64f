"""Generates zplans.inc: the compile-time z-axis FFT plans of the fused z pass.

For every 5-smooth line length 2 <= N <= 512 it picks, among the radix
sequences with the fewest stages (register radices 2..16), the sequence and the
padded layout that minimise a cost of shared-memory wavefronts plus issued
instructions of one three-line warp task (forward transform, spectral product,
inverse transform).

Layout: element idx = q * R_last + r of a line lives at q * S + r (S >= R_last),
so every butterfly of every stage reads its R elements at one base address plus
compile-time offsets; lines are LW elements apart.

Bank model: 32 banks of 4 bytes; 8-byte accesses are served per half-warp and
a group takes as many wavefronts as the largest number of distinct words in one
bank (this reproduces the shared-memory wavefront counts ncu reports).

Usage: python gen_zplans.py > zplans.inc
"""
import sys

RADICES = (16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2)
NL = 3          # component lines per warp task
ESIZE = 8       # complex FP32


def smooth(n):
    for p in (2, 3, 5):
        while n % p == 0:
            n //= p
    return n == 1


def sequences(n):
    out = []

    def rec(rem, cur, depth):
        if rem == 1:
            out.append(tuple(cur))
            return
        if depth == 0:
            return
        for r in RADICES:
            if rem % r == 0:
                rec(rem // r, cur + [r], depth - 1)
    for depth in range(1, 10):
        rec(n, [], depth)
        if out:
            return [s for s in out if len(s) == depth]
    return []


def wavefronts(addrs):
    group = 128 // ESIZE
    wpe = ESIZE // 4
    total = 0
    for g0 in range(0, len(addrs), group):
        banks = {}
        for a in addrs[g0:g0 + group]:
            for k in range(wpe):
                w = a * wpe + k
                banks.setdefault(w & 31, set()).add(w)
        total += max(len(v) for v in banks.values())
    return total


def dft_cost(r):
    base = {2: 4, 3: 12, 4: 16, 5: 34, 8: 52}
    if r in base:
        return base[r]
    a, b = {6: (2, 3), 9: (3, 3), 10: (2, 5), 12: (4, 3), 15: (3, 5), 16: (4, 4)}[r]
    return a * dft_cost(b) + b * dft_cost(a) + 4 * (a - 1) * (b - 1)


def cost(n, rad, S, LW):
    rl = rad[-1]

    def addr(idx):
        return (idx // rl) * S + idx % rl
    wf = 0
    instr = 0
    Ls = n
    for s, R in enumerate(rad):
        M = Ls // R
        B = n // R
        T = NL * B
        for t0 in range(0, T, 32):
            chunk = range(t0, min(T, t0 + 32))
            for i in range(R):
                a = []
                for t in chunk:
                    j, u = divmod(t, B)
                    b, n1 = divmod(u, M)
                    a.append(j * LW + addr(b * Ls + n1 + i * M))
                wf += 2 * wavefronts(a)                       # load + store
            instr += 2 * R + dft_cost(R) + (5 * (R - 1) if M > 1 else 0) + 16
        Ls = M
    wf *= 2                                                       # forward + inverse
    instr *= 2
    for j in range(NL):                                           # load, product (2), store
        for z0 in range(0, n, 32):
            wf += 4 * wavefronts([j * LW + addr(z) for z in range(z0, min(n, z0 + 32))])
    return wf + instr / 4.0


def choose(n):
    best = None
    for rad in sequences(n):
        rl = rad[-1]
        for S in range(rl, rl + 4):
            top = (n // rl - 1) * S + rl
            for d in range(16):
                LW = top + d
                c = cost(n, rad, S, LW)
                key = (c, LW, S)
                if best is None or key < best[0]:
                    best = (key, rad, S, LW)
    return best[1], best[2], best[3]


def main():
    lines = ["// Generated by gen_zplans.py: compile-time z-axis plans of the fused z pass.",
             "// BDDA_ZPLAN(index, N, S, LW, radices...): element q*R_last + r at q*S + r, lines LW apart."]
    idx = 0
    for n in range(2, 513):
        if not smooth(n):
            continue
        rad, S, LW = choose(n)
        lines.append("BDDA_ZPLAN(%d, %d, %d, %d, %s)" % (idx, n, S, LW, ", ".join(str(r) for r in rad)))
        idx += 1
        print(n, rad, S, LW, file=sys.stderr, flush=True)
    print("\n".join(lines))


if __name__ == "__main__":
    main()

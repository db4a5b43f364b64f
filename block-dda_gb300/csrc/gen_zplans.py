"""Generates the compile-time FFT plans of the block-MVP passes.

  zplans.inc  three-line plans of the complex FP32 fused z pass (one warp
              transforms the three component lines of an (x, y, rhs) task);
              the first stage may take a radix up to 32, and a last radix
              <= FUSED_MAX lets the last forward stage, the Green product and
              the first inverse stage run as one step (sfft::middle3), so
              that a 2-stage plan makes two shared-memory round trips per
              line triple instead of four or more
  zwplans.inc three-line plans of the 16-byte z passes (FP64 / double-float:
              register radices <= 16, no fused step)
  tplans.inc  single-line plans of the strided x / y passes (one warp per
              line, eight lines per CTA filled and drained as a tile)

For every 5-smooth line length 2 <= N <= 512 it picks, among the radix
sequences with the fewest or one more than the fewest stages (register
radices 2..16, and the first-stage radices of zplans.inc), the sequence and
the padded layout that minimise a cost of shared-memory wavefronts plus
issued instructions per line.

Layout: element idx = q * R_last + r of a line lives at q * S + r (S >= R_last),
so every butterfly of every stage reads its R elements at one base address plus
compile-time offsets; lines are LW elements apart.

Bank model: 32 banks of 4 bytes; 8-byte accesses are served per half-warp and
a group takes as many wavefronts as the largest number of distinct words in one
bank (this reproduces the shared-memory wavefront counts ncu reports).

  yplans.inc  the column-pair y passes (two lines interleaved element by
              element per warp): the radix sequences of tplans.inc, the
              padded layout chosen for the interleaved pairs and the 16-byte
              tile fill / drain of eight column pairs

Usage: python gen_zplans.py [z] [zw] [t] [il]   (writes the tables beside it;
       il reads the radix sequences from tplans.inc)
"""
import os
import sys

RADICES = (16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2)
FIRST_RADICES = (32, 30, 27, 25, 24, 20, 18) + RADICES   # first stage of the complex FP32 z plans
FUSED_MAX = 10  # largest last radix of the fused middle step (kFusedMaxRadix)
Z_MAX_PAD = 1.2  # line pitch of the complex FP32 z plans at most 1.2 N + 2
ESIZE = 8       # complex FP32


def smooth(n):
    for p in (2, 3, 5):
        while n % p == 0:
            n //= p
    return n == 1


def sequences(n, first=RADICES):
    """Radix sequences with the fewest stages and with one more (first: the
    radices the first stage may take)."""
    out = {}

    def rec(rem, cur, depth):
        if rem == 1:
            out.setdefault(len(cur), []).append(tuple(cur))
            return
        if depth == 0:
            return
        for r in (first if not cur else RADICES):
            if rem % r == 0:
                rec(rem // r, cur + [r], depth - 1)
    for depth in range(1, 12):
        rec(n, [], depth)
        if out:
            break
    m = min(out)
    out = {}
    rec(n, [], m + 1)
    return out.get(m, []) + out.get(m + 1, [])


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
    a, b = {6: (2, 3), 9: (3, 3), 10: (2, 5), 12: (4, 3), 15: (3, 5), 16: (4, 4), 18: (2, 9), 20: (4, 5),
            24: (8, 3), 25: (5, 5), 27: (3, 9), 30: (2, 15), 32: (4, 8)}[r]
    return a * dft_cost(b) + b * dft_cost(a) + 4 * (a - 1) * (b - 1)


def stage_cost(n, rad, S, LW, NL):
    """Wavefronts and warp instructions of one transform of NL lines."""
    rl = rad[-1]

    def addr(idx):
        return (idx // rl) * S + idx % rl
    wf = 0
    instr = 0
    Ls = n
    for R in rad:
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
    return wf, instr


def cost_z(n, rad, S, LW):
    """One three-line task: forward, product, inverse."""
    rl = rad[-1]
    wf, instr = stage_cost(n, rad, S, LW, 3)
    wf, instr = 2 * wf, 2 * instr
    for j in range(3):                                            # load, product (2), store
        for z0 in range(0, n, 32):
            wf += 4 * wavefronts([j * LW + (z // rl) * S + z % rl for z in range(z0, min(n, z0 + 32))])
    return wf + instr / 4.0


def stage_pass(n, rad, S, LW, s, NL, load, store):
    """Wavefronts and warp instructions of stage s of NL lines (one warp)."""
    rl = rad[-1]
    Ls = n
    for R in rad[:s]:
        Ls //= R
    R = rad[s]
    M = Ls // R
    B = n // R
    T = NL * B
    wf = instr = 0
    for t0 in range(0, T, 32):
        chunk = range(t0, min(T, t0 + 32))
        for i in range(R):
            a = []
            for t in chunk:
                j, u = divmod(t, B)
                b, n1 = divmod(u, M)
                idx = b * Ls + n1 + i * M
                a.append(j * LW + (idx // rl) * S + idx % rl)
            wf += (load + store) * wavefronts(a)
        instr += (load + store) * R + dft_cost(R) + (5 * (R - 1) if M > 1 else 0) + 16
    return wf, instr


def cost_zf(n, rad, S, LW):
    """One three-line task of the complex FP32 z pass: the first forward
    stage reads global memory and the last inverse stage writes it (shared
    memory stores / loads only); with nst >= 2 and a last radix <= FUSED_MAX
    the last forward stage, the product and the first inverse stage are one
    step in which a thread takes one butterfly of all three lines."""
    rl, nst = rad[-1], len(rad)
    fused = nst >= 2 and rl <= FUSED_MAX
    wf = instr = 0
    for s in range(nst - 1 if fused else nst):
        w, i = stage_pass(n, rad, S, LW, s, 3, 0 if s == 0 else 1, 1)   # forward
        wf, instr = wf + w, instr + i
        w, i = stage_pass(n, rad, S, LW, s, 3, 1, 0 if s == 0 else 1)   # inverse
        wf, instr = wf + w, instr + i
    if fused:
        B = n // rl
        for b0 in range(0, B, 32):
            for j in range(3):
                for i in range(rl):
                    wf += 2 * wavefronts([j * LW + b * S + i for b in range(b0, min(B, b0 + 32))])
            instr += 6 * rl + 2 * dft_cost(rl) * 3 + rl * (12 + 36) + 16
    else:
        for j in range(3):                                            # product: load, store
            for z0 in range(0, n, 32):
                wf += 2 * wavefronts([j * LW + (z // rl) * S + z % rl for z in range(z0, min(n, z0 + 32))])
        instr += ((n + 31) // 32) * (6 + 12 + 36)
    return wf + instr / 4.0


def cost_tile(n, rad, S, LW):
    """One line of a tile pass: one transform plus its share of the tile fill and drain."""
    rl = rad[-1]
    wf, instr = stage_cost(n, rad, S, LW, 1)
    tw = 0
    for i0 in range(0, 8 * n, 32):
        tw += wavefronts([((i0 + l) & 7) * LW + ((((i0 + l) >> 3) // rl) * S + ((i0 + l) >> 3) % rl)
                          for l in range(min(32, 8 * n - i0))])
    return wf + instr / 4.0 + 2 * tw / 8.0


def wavefronts16(chunks):
    """16-byte accesses, served per quarter-warp: a group of eight takes as many
    wavefronts as the most distinct 16-byte chunks on one set of four banks."""
    total = 0
    for g0 in range(0, len(chunks), 8):
        groups = {}
        for c in chunks[g0:g0 + 8]:
            groups.setdefault(c & 7, set()).add(c)
        total += max(len(v) for v in groups.values())
    return total


def stage_cost_il(n, rad, S, LW):
    """Shared-memory wavefronts of one transform of a line pair interleaved
    element by element (element idx of line h at 8-byte word 2 addr(idx) + h;
    lane t handles butterfly t >> 1 of line t & 1)."""
    rl = rad[-1]

    def addr(idx):
        return (idx // rl) * S + idx % rl
    wf = 0
    Ls = n
    for R in rad:
        M = Ls // R
        B = n // R
        for t0 in range(0, 2 * B, 32):
            chunk = range(t0, min(2 * B, t0 + 32))
            for i in range(R):
                a = []
                for t in chunk:
                    b, n1 = divmod(t >> 1, M)
                    a.append(2 * addr(b * Ls + n1 + i * M) + (t & 1))
                wf += 2 * wavefronts(a)                       # load + store
        Ls = M
    return wf


def cost_y_il(n, rad, S, LW):
    """One line pair of a column-pair y pass (k_pass_y2i): its transform plus
    its share of the tile fill and drain, where the eight lanes of a
    quarter-warp move one row of the task's eight column pairs (pair p of row
    r at 16-byte chunk p LW + addr(r)), over the n rows of the padded line."""
    rl = rad[-1]
    tw = 0
    for r in range(n):
        a = (r // rl) * S + r % rl
        tw += wavefronts16([p * LW + a for p in range(8)])
    return stage_cost_il(n, rad, S, LW) + 2 * tw / 8.0


def choose_layout(n, rad, cost):
    """The padded layout (S, LW) for a fixed radix sequence."""
    rl = rad[-1]
    best = None
    for S in range(rl, rl + 4):
        top = (n // rl - 1) * S + rl
        for d in range(16):
            LW = top + d
            key = (cost(n, rad, S, LW), LW, S)
            if best is None or key < best[0]:
                best = (key, S, LW)
    return best[1], best[2]


def choose(n, cost, first=RADICES, max_pad=None):
    """Radix sequence and layout of least cost; max_pad caps the line pitch
    at n * max_pad + 2 elements (shared memory per warp sets the occupancy,
    which the per-task cost does not see)."""
    best = None
    for rad in sequences(n, first):
        rl = rad[-1]
        for S in range(rl, rl + 4):
            top = (n // rl - 1) * S + rl
            for d in range(16):
                LW = top + d
                if max_pad is not None and LW > n * max_pad + 2:
                    continue
                key = (cost(n, rad, S, LW), LW, S)
                if best is None or key < best[0]:
                    best = (key, rad, S, LW)
    return best[1], best[2], best[3]


FUSED_WIDE_MIN_N = 181  # kFusedWideMinN: shorter z lines keep the packed-pair kernel's plans


def z_entry(n):
    """Plan of the complex FP32 z table.  Lines shorter than FUSED_WIDE_MIN_N
    (the packed-pair z pass's range: three 8-warp CTAs of it fit up to a
    pitch of ~200) keep the 16-byte table's plan (cost_z, radices <= 16, a
    fused step only up to radix 5), on which the packed kernel was measured
    faster than the two-stage fused plans (N=16384, Pz=150: packed 10 x 15
    0.64 ms, pipelined 15 x 10 0.76 ms); longer lines take the two-stage fused
    model (cost_zf, first-stage radices up to 32)."""
    if n < FUSED_WIDE_MIN_N:
        return choose(n, cost_z)
    return choose(n, cost_zf, FIRST_RADICES, Z_MAX_PAD)


def write(path, macro, what, cost, first=RADICES, max_pad=None, entry=None):
    lines = ["// Generated by gen_zplans.py: compile-time plans of the %s." % what,
             "// %s(index, N, S, LW, radices...): element q*R_last + r at q*S + r, lines LW apart." % macro]
    idx = 0
    for n in range(2, 513):
        if not smooth(n):
            continue
        rad, S, LW = entry(n) if entry else choose(n, cost, first, max_pad)
        lines.append("%s(%d, %d, %d, %d, %s)" % (macro, idx, n, S, LW, ", ".join(str(r) for r in rad)))
        idx += 1
        print(macro, n, rad, S, LW, file=sys.stderr, flush=True)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_radices(path, macro):
    """{N: radices} of a generated table."""
    out = {}
    with open(path) as f:
        for line in f:
            if line.startswith(macro + "("):
                v = [int(x) for x in line[len(macro) + 1:line.index(")")].split(",")]
                out[v[1]] = tuple(v[4:])
    return out


def write_il(path, macro, what, cost, radices):
    """A table with the given radix sequences and the layout of `cost`."""
    lines = ["// Generated by gen_zplans.py: compile-time plans of the %s." % what,
             "// %s(index, N, S, LW, radices...): element q*R_last + r at q*S + r, lines LW apart." % macro]
    for idx, n in enumerate(sorted(radices)):
        rad = radices[n]
        S, LW = choose_layout(n, rad, cost)
        lines.append("%s(%d, %d, %d, %d, %s)" % (macro, idx, n, S, LW, ", ".join(str(r) for r in rad)))
        print(macro, n, rad, S, LW, file=sys.stderr, flush=True)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    which = sys.argv[1:] or ["z", "t"]
    if "il" in which:
        # the column-pair y passes: the radix sequences of the single-line
        # table (they fix the digit order the Green spectrum is packed in),
        # the layout for interleaved line pairs and 16-byte rows of eight
        # pairs.  (The x passes drain two rows of four pairs per quarter-warp;
        # modelled the same way, tplans.inc's layouts are already as good
        # there, so they keep that table.)
        rad = read_radices(os.path.join(here, "tplans.inc"), "BDDA_TPLAN")
        write_il(os.path.join(here, "yplans.inc"), "BDDA_YPLAN",
                 "column-pair y passes (line pairs interleaved, eight pairs per task)", cost_y_il, rad)
        return
    if "z" in which:
        write(os.path.join(here, "zplans.inc"), "BDDA_ZPLAN", "complex FP32 fused z pass (three lines per warp)",
              cost_zf, entry=z_entry)
    if "zw" in which:
        write(os.path.join(here, "zwplans.inc"), "BDDA_ZWPLAN",
              "16-byte (FP64 / double-float) z passes (three lines per warp)", cost_z)
    if "t" in which:
        write(os.path.join(here, "tplans.inc"), "BDDA_TPLAN", "strided x / y passes (one line per warp)",
              cost_tile)


if __name__ == "__main__":
    main()

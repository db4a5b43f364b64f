"""The generated compile-time plan tables (CPU).

* yplans.inc (column-pair y passes) lists the same lengths with the same radix
  sequences as tplans.inc: the sequence fixes the digit order of a transform,
  and the Green spectrum is packed in the order of the runtime plans, which
  take their sequences from tplans.inc;
* every layout holds its line: element q R_last + r at q S + r with
  S >= R_last, so the last element sits below the pitch LW;
* the generator reproduces the committed yplans.inc, and the complex FP32 z
  table's entries for the default workload's lengths;
* only the first stage of a complex FP32 z plan takes a radix above 16 (the
  register radices of every other kernel), the 16-byte z table none, and both
  z tables list the same lengths.
"""
import importlib.util
import os

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "block-dda_gb300", "csrc")


def _table(name, macro):
    out = {}
    with open(os.path.join(CSRC, name)) as f:
        for line in f:
            if line.startswith(macro + "("):
                v = [int(x) for x in line[len(macro) + 1:line.index(")")].split(",")]
                out[v[1]] = (v[2], v[3], tuple(v[4:]))
    return out


def _gen():
    spec = importlib.util.spec_from_file_location("gen_zplans", os.path.join(CSRC, "gen_zplans.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_y_table_keeps_the_radix_sequences():
    t = _table("tplans.inc", "BDDA_TPLAN")
    y = _table("yplans.inc", "BDDA_YPLAN")
    assert sorted(t) == sorted(y)
    for n in t:
        assert t[n][2] == y[n][2], n


@pytest.mark.parametrize("name,macro", [("zplans.inc", "BDDA_ZPLAN"), ("zwplans.inc", "BDDA_ZWPLAN"),
                                        ("tplans.inc", "BDDA_TPLAN"), ("yplans.inc", "BDDA_YPLAN")])
def test_layouts_hold_their_lines(name, macro):
    tab = _table(name, macro)
    assert tab
    for n, (S, LW, rad) in tab.items():
        prod = 1
        for r in rad:
            prod *= r
        assert prod == n, (name, n, rad)
        rl = rad[-1]
        assert S >= rl, (name, n)
        last = ((n - 1) // rl) * S + (n - 1) % rl
        assert last < LW, (name, n, S, LW)


def test_generator_reproduces_the_y_table(tmp_path):
    g = _gen()
    rad = g.read_radices(os.path.join(CSRC, "tplans.inc"), "BDDA_TPLAN")
    out = tmp_path / "yplans.inc"
    g.write_il(str(out), "BDDA_YPLAN", "column-pair y passes (line pairs interleaved, eight pairs per task)",
               g.cost_y_il, rad)
    with open(os.path.join(CSRC, "yplans.inc")) as f:
        assert out.read_text() == f.read()


def test_z_tables_radix_limits():
    z = _table("zplans.inc", "BDDA_ZPLAN")
    zw = _table("zwplans.inc", "BDDA_ZWPLAN")
    assert sorted(z) == sorted(zw)
    for n, (_, _, rad) in z.items():
        assert rad[0] <= 32 and all(r <= 16 for r in rad[1:]), (n, rad)
    for n, (_, _, rad) in zw.items():
        assert all(r <= 16 for r in rad), (n, rad)
    # the default workload's z length: two stages, fused last radix
    assert z[250][2] == (25, 10) and z[243][2] == (27, 9)
    # lines shorter than the two-stage threshold (the packed-pair kernel's range) keep the 16-byte plans
    g = _gen()
    for n in z:
        if n < g.FUSED_WIDE_MIN_N:
            assert z[n] == zw[n], n


@pytest.mark.parametrize("n", [125, 150, 243, 250])
def test_generator_reproduces_z_entries(n):
    g = _gen()
    rad, S, LW = g.z_entry(n)
    assert _table("zplans.inc", "BDDA_ZPLAN")[n] == (S, LW, tuple(rad))
    if n <= 150:   # packed-pass lengths keep the 16-byte table's plan
        assert _table("zwplans.inc", "BDDA_ZWPLAN")[n] == (S, LW, tuple(rad))


def test_generator_constants_match_the_kernels():
    """The generator's fused-step rule is the kernels' (fused_z, mvp.hpp)."""
    import re
    g = _gen()
    src = open(os.path.join(CSRC, "mvp.hpp")).read()
    const = {k: int(v) for k, v in re.findall(r"constexpr int (k\w+) = (\d+);", src)}
    assert const["kFusedMaxRadix"] == g.FUSED_MAX
    assert const["kFusedWideMinN"] == g.FUSED_WIDE_MIN_N

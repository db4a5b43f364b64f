"""The generated compile-time plan tables (CPU).

* yplans.inc (column-pair y passes) lists the same lengths with the same radix
  sequences as tplans.inc: the sequence fixes the digit order of a transform,
  and the Green spectrum is packed in the order of the runtime plans, which
  take their sequences from tplans.inc;
* every layout holds its line: element q R_last + r at q S + r with
  S >= R_last, so the last element sits below the pitch LW;
* the generator reproduces the committed yplans.inc.
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


@pytest.mark.parametrize("name,macro", [("zplans.inc", "BDDA_ZPLAN"), ("tplans.inc", "BDDA_TPLAN"),
                                        ("yplans.inc", "BDDA_YPLAN")])
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

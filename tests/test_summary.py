"""The sweep summary (the notebook's speed-up table without pandas) on synthetic result
trees in the driver's layout and in the library's bare Results layout."""
from __future__ import annotations

import os

import pytest

from gpu4snn_gb300 import summary as S


def _write(root, gpu, it, mode, alg, e, ewd, spk, n=2500, nsyn=1000):
    parts = [root] + ([gpu, str(it)] if gpu else []) + ["Results", f"N{n}Nsyn{nsyn}Regime{mode}Alg{alg}"]
    d = os.path.join(*parts)
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "sim_overview.csv"), "w") as f:  # no trailing newline, as the reference
        f.write(f"N elapsed(ms) elapsedwithdata(ms) totalspkcount\n{n} {e} {ewd} {spk}")


def test_speedup_table_matches_the_notebook_definition(tmp_path):
    root = str(tmp_path)
    t = {0: 40.0, 1: 90.0, 2: 60.0, 3: 20.0, 4: 10.0}
    for it in (2000, 10000):
        for mode in (0, 1, 2):
            for alg, e in t.items():
                _write(root, "GB300", it, mode, alg, e * it / 2000, 2 * e * it / 2000 + 5, 1000 + alg)
    runs = S.collect(root)
    assert len(runs) == 30 and runs[0].gpu == "GB300"
    rows = S.speedup_table(runs)
    assert len(rows) == 2 * 2 * 3 * 2  # modes 1,2 x new SKL,AB x old AP,N,S x iterations
    r = next(r for r in rows if r[1] == 2000 and r[2] == 1 and r[3] == "N" and r[4] == "SKL")
    assert r[5] == 185.0 and r[6] == 25.0 and r[7] == pytest.approx(7.4) and r[8] == "Y"
    assert r[9] == 1001 and r[10] == 1004
    rows_k = S.speedup_table(runs, metric="elapsed", modes=(2,))
    assert all(x[2] == 2 for x in rows_k)
    r = next(r for r in rows_k if r[1] == 10000 and r[3] == "AP" and r[4] == "AB")
    assert r[7] == pytest.approx(2.0)
    g = S.mean_speedups(rows_k)
    assert g[("SKL", "N")] == pytest.approx(9.0)


def test_bare_results_layout_and_cli(tmp_path, capsys):
    root = str(tmp_path)
    _write(root, "", 0, 1, 4, 5.0, 6.0, 10)
    _write(root, "", 0, 1, 0, 50.0, 60.0, 11)
    runs = S.collect(root)
    assert [(r.gpu, r.iterations) for r in runs] == [("", 0), ("", 0)]
    out = str(tmp_path / "t.csv")
    assert S.main([root, "--modes", "1", "--csv", out]) == 0
    lines = open(out).read().splitlines()
    assert lines[0].startswith("GPU,Iterations,Mode,Old Alg.,New Alg.")
    assert len(lines) == 2 and ",AP,SKL,60.0,6.0,10.0,Y,11,10" in lines[1]
    assert "SKL over AP: geometric-mean speed-up 10.00" in capsys.readouterr().out


def test_read_overview_rejects_other_files(tmp_path):
    p = tmp_path / "sim_overview.csv"
    p.write_text("x y\n1 2")
    with pytest.raises(ValueError):
        S.read_overview(str(p))

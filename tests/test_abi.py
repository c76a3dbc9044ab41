"""CPU tests of the C ABI boundary: the library loads, exports every entry point the
header declares, validates its inputs before touching the GPU, and its host-side table
generator reproduces the reference's own tables."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(g4s_\w+)\s*\(", text))
    return names


def test_header_symbols_exported(g4s):
    from gpu4snn_gb300 import _lib
    lib = C.CDLL(_lib.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    bound = {s[0] for s in _lib.SIGNATURES}
    assert names <= bound, sorted(names - bound)


def test_abi_version(g4s):
    assert g4s.load().g4s_abi_version() == 1


def test_invalid_descriptors_rejected(g4s):
    from gpu4snn_gb300 import _lib
    bad = [dict(n=1, nsyn=1), dict(n=100, nsyn=100), dict(n=100, nsyn=0), dict(n=100, nsyn=10, exc_permille=1200),
           dict(n=100, nsyn=10, conn_law=7), dict(n=100, nsyn=10, drive_scale=float("nan"))]
    for kw in bad:
        with pytest.raises(g4s.G4SError) as e:
            g4s.Network(**kw)
        assert e.value.code == _lib.ERR_INVALID, kw


def test_null_arguments(g4s):
    L = g4s.load()
    assert L.g4s_net_create(None, None) == -1
    assert L.g4s_net_run(None, 1, 4) == -1
    assert b"null" in L.g4s_last_error()
    assert L.g4s_inject_fault(None, 99) == -1


@pytest.mark.parametrize("fn", ["ref_tables_N20_S5_seed7.npz", "ref_tables_N200_S50_seed3.npz",
                                "ref_tables_N101_S101_seed11.npz"])
def test_library_glibc_tables_match_reference(g4s, fn):
    g = np.load(os.path.join(GOLDEN, fn))
    n, nsyn = g["idx"].shape
    seed = int(fn.split("seed")[1].split(".")[0])
    idx, w = g4s.conn_glibc(seed, n, nsyn, stride=nsyn)
    assert np.array_equal(idx, g["idx"]) and np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
    idx4, w4 = g4s.conn_glibc(seed, n, nsyn)
    assert np.array_equal(idx4[:, :nsyn], g["idx"]) and (idx4[:, nsyn:] == -1).all()


def test_library_glibc_tables_reference_size(g4s, oracle):
    import hashlib
    import json
    rec = json.load(open(os.path.join(GOLDEN, "ref_tables_digest.json")))[0]
    idx, w = g4s.conn_glibc(rec["seed"], rec["n"], rec["nsyn"], stride=rec["nsyn"])
    h = hashlib.sha256()
    h.update(idx.tobytes())
    h.update(w.tobytes())
    assert h.hexdigest() == rec["sha256"]


def test_driver_cli_parses(monkeypatch, tmp_path):
    from gpu4snn_gb300 import gpu4snn as drv
    calls = []

    def fake(n, nsyn, it, alg, mode, seed, conn, root):
        calls.append((n, nsyn, it, alg, mode, seed, conn))
        os.makedirs(os.path.join(root, "Results", "x"), exist_ok=True)

    monkeypatch.setattr(drv, "run_protocol", fake)
    monkeypatch.chdir(tmp_path)
    assert drv.main(["Quadro", "2000"]) == 0
    assert calls[-1] == (2500, 1000, 2000, -1, -1, 1, 0)
    assert os.path.isdir(tmp_path / "Quadro" / "2000" / "Results" / "x")
    drv.main(["B", "10", "--N", "100", "--Nsyn", "10", "--algorithm", "SKL", "--mode", "2", "--conn", "glibc"])
    assert calls[-1] == (100, 10, 10, 4, 2, 1, 1)

"""g4s_run_noalloc, the allocation-free entry point, against g4s_net_run.

The entry point exists for callers that cannot allocate device memory while they step a
network (real-time loops that cannot take an allocation's device-wide synchronisation,
hosts whose device memory is a capped pool): it runs the SKL team kernel on device arrays
the caller owns and keeps its own scratch in a fixed device array.  Here the caller's
arrays are torch tensors built from a handle's initial state and sorted tables; two calls
in a row must give exactly the rasters, states and pending currents of two g4s_net_run
calls on an identical handle.  The cases cover one CTA, a two-CTA team, and a team of 8
at the 131072-neuron limit driven hard enough that a step's spikes overflow the rank's
shared-memory window (the tagged dense-list path, whose words the second call must find
cleared).  This file is collected last so that a failure here cannot hide the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class DevNet(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("nexc", C.c_int64), ("nsyn", C.c_int32), ("stride", C.c_int32),
        ("seed", C.c_uint64), ("ge", C.c_float), ("gi", C.c_float),
        ("vu", C.c_void_p), ("abcd", C.c_void_p), ("acc", C.c_void_p), ("i_last", C.c_void_p),
        ("spike_stat", C.c_void_p), ("idx", C.c_void_p), ("w", C.c_void_p),
    ]


def _raster(counts, base, raster, t0):
    t, ids = [], []
    for lt, (c, b) in enumerate(zip(counts, base)):
        t.append(np.full(c, t0 + lt, dtype=np.int32))
        ids.append(np.sort(raster[b:b + c]))
    return np.concatenate(t), np.concatenate(ids)


@pytest.mark.parametrize("n,nsyn,team,drive", [(20000, 300, 2, 1.0), (6000, 1000, 1, 1.0), (131072, 100, 8, 2.0)])
def test_noalloc_matches_net_run(g4s, n, nsyn, team, drive):
    torch = pytest.importorskip("torch")
    from gpu4snn_gb300 import _lib
    L = _lib.load()
    seed, steps, dev = 41, 60, "cuda:0"
    with g4s.Network(n, nsyn, seed=seed, drive_scale=drive) as ref, \
            g4s.Network(n, nsyn, seed=seed, drive_scale=drive) as src:
        st = src.state()
        idx, w = src.tables()
        vu = torch.tensor(np.stack([st["v"], st["u"]], 1), device=dev)
        abcd = torch.tensor(np.stack([st["a"], st["b"], st["c"], st["d"]], 1), device=dev)
        acc = torch.zeros(n, dtype=torch.int64, device=dev)
        ilast = torch.zeros(n, dtype=torch.float32, device=dev)
        sstat = torch.zeros((n, 8), dtype=torch.int32, device=dev)
        sstat[:, 1] = -1
        tidx = torch.tensor(idx, device=dev)
        tw = torch.tensor(w, device=dev)
        counts = torch.zeros(steps, dtype=torch.int32, device=dev)
        base = torch.zeros(steps, dtype=torch.int64, device=dev)
        raster = torch.zeros(n * steps, dtype=torch.int32, device=dev)
        status = torch.ones(1, dtype=torch.int32, device=dev)
        d = DevNet(n=n, nexc=n * 800 // 1000, nsyn=nsyn, stride=idx.shape[1], seed=seed,
                   ge=float(np.float32(5.0) * np.float32(drive)), gi=float(np.float32(2.0) * np.float32(drive)),
                   vu=vu.data_ptr(), abcd=abcd.data_ptr(), acc=acc.data_ptr(), i_last=ilast.data_ptr(),
                   spike_stat=sstat.data_ptr(), idx=tidx.data_ptr(), w=tw.data_ptr())
        torch.cuda.synchronize()
        for call in range(2):
            rc = L.g4s_run_noalloc(C.byref(d), call * steps, steps, team, call, counts.data_ptr(), base.data_ptr(),
                                   raster.data_ptr(), n * steps, status.data_ptr(), None)
            assert rc == 0, L.g4s_last_error()
            torch.cuda.synchronize()
            assert int(status.item()) == 0
            ref.run(steps, g4s.ALG_SKL)
            rt, rid = ref.raster()
            sel = rt >= call * steps
            if team == 8:
                # the case exists for the dense-list path: a step with more spikes than the
                # rank's shared-memory window (1728 ids at 16384 neurons per CTA)
                assert np.bincount(rt[sel] - call * steps).max() > 1728
            t, ids = _raster(counts.cpu().numpy(), base.cpu().numpy(), raster.cpu().numpy(), call * steps)
            assert np.array_equal(t, rt[sel]) and np.array_equal(ids, rid[sel])
        s = ref.state()
        got = vu.cpu().numpy()
        assert np.array_equal(got[:, 0].view(np.uint32), s["v"].view(np.uint32))
        assert np.array_equal(got[:, 1].view(np.uint32), s["u"].view(np.uint32))
        assert np.array_equal(ilast.cpu().numpy().view(np.uint32), s["I"].view(np.uint32))
        assert np.array_equal(sstat.cpu().numpy()[:, 0], s["nospks"])
        assert np.array_equal(acc.cpu().numpy(), ref.currents())


def test_noalloc_rejects_oversize(g4s):
    from gpu4snn_gb300 import _lib
    L = _lib.load()
    d = DevNet(n=200000, nexc=160000, nsyn=10, stride=12, seed=1, ge=5.0, gi=2.0, vu=1, abcd=1, acc=1,
               i_last=1, spike_stat=1, idx=1, w=1)
    assert L.g4s_run_noalloc(C.byref(d), 0, 1, 8, 0, 1, 1, None, 0, None, None) == _lib.ERR_INVALID
    assert b"131072" in L.g4s_last_error()
    d.n, d.nexc = 100000, 80000
    assert L.g4s_run_noalloc(C.byref(d), 0, 1, 4, 0, 1, 1, None, 0, None, None) == _lib.ERR_INVALID
    assert b"per CTA" in L.g4s_last_error()

"""Regenerate the golden fixtures of this directory.

    python tests/golden/make_golden.py

philox_kat.json      Philox4x64-10 blocks from numpy.random.Philox (numpy increments the
                     counter before each block: block k of a generator created with
                     counter c is Philox(c + k + 1)).
philox4x32_kat.json  Philox4x32-10 blocks from the CUDA toolkit's cuRAND host generator.
ref_tables_*.npz     connectivity tables produced by the reference's own host code
                     (gpu4snn.cu:873-898), built and run by `make -C oracle ref` with the
                     seed fixed through the wrapped time() call.
ref_tables_digest.json  SHA-256 of the reference's tables at its notebook size (N=2500,
                     Nsyn=1000) for three seeds, plus their first rows.
oracle_small.json    a regression record of the oracle itself (raster digest, spike count,
                     final v digest) for a small network, to catch unintended drift.
"""
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import g4s_oracle as O  # noqa: E402

KAT_CASES = [
    ([0, 0], [0, 0, 0, 0]),
    ([0, 0], [5, 7, 9, 11]),
    ([123456789, 987654321], [0, 0, 0, 0]),
    ([2**64 - 1, 5], [2**64 - 2, 3, 0, 0]),
    ([0xDEADBEEF, 0x1234567890ABCDEF], [2**63, 2**63 + 1, 2**62, 7]),
    ([1, 4], [99, 1000, 2, 0]),
]


def kat():
    out = []
    for key, ctr in KAT_CASES:
        bg = np.random.Philox(counter=np.array(ctr, dtype=np.uint64), key=np.array(key, dtype=np.uint64))
        blocks = bg.random_raw(12).reshape(3, 4)
        out.append({"key": [str(k) for k in key], "counter": [str(c) for c in ctr],
                    "blocks": [[str(int(x)) for x in b] for b in blocks]})
    return out


def kat32():
    """Philox4x32-10 blocks from the CUDA toolkit's cuRAND host generator (a library run,
    no GPU needed): block k of seed s is Philox4x32-10(counter (0, 0, k, 0), key (s_lo, s_hi))."""
    import ctypes as C
    lib = None
    for path in ("/usr/local/cuda/lib64/libcurand.so", "libcurand.so", "libcurand.so.10"):
        try:
            lib = C.CDLL(path)
            break
        except OSError:
            continue
    if lib is None:
        raise SystemExit("libcurand not found")
    PHILOX = 161  # CURAND_RNG_PSEUDO_PHILOX4_32_10 (curand.h)
    out = []
    for seed in (0, 1, 0x123456789ABCDEF, 2**64 - 1, 0xFEEDFACE):
        g = C.c_void_p()
        assert lib.curandCreateGeneratorHost(C.byref(g), PHILOX) == 0
        assert lib.curandSetPseudoRandomGeneratorSeed(g, C.c_ulonglong(seed)) == 0
        buf = (C.c_uint * 16)()
        assert lib.curandGenerate(g, buf, 16) == 0
        lib.curandDestroyGenerator(g)
        out.append({"seed": str(seed), "blocks": [[int(buf[4 * k + j]) for j in range(4)] for k in range(4)]})
    return out


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main():
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump(kat(), f, indent=1)
    with open(os.path.join(HERE, "philox4x32_kat.json"), "w") as f:
        json.dump(kat32(), f, indent=1)
    if not os.path.exists(O.REF_TABLES):
        raise SystemExit("build the reference's table generator first: make -C oracle ref")
    with tempfile.TemporaryDirectory() as tmp:
        for n, nsyn, seed in [(20, 5, 7), (200, 50, 3), (101, 101, 11)]:
            idx, w = O.ref_tables(seed, n, nsyn, tmp)
            np.savez_compressed(os.path.join(HERE, f"ref_tables_N{n}_S{nsyn}_seed{seed}.npz"), idx=idx, w=w)
        big = []
        for seed in (1, 2, 1796309881):
            idx, w = O.ref_tables(seed, 2500, 1000, tmp)
            big.append({"seed": seed, "n": 2500, "nsyn": 1000, "sha256": digest(idx, w),
                        "row0_idx": idx[0, :16].tolist(), "row0_w_bits": w[0, :16].view(np.uint32).tolist(),
                        "last_row_idx": idx[-1, :16].tolist()})
        with open(os.path.join(HERE, "ref_tables_digest.json"), "w") as f:
            json.dump(big, f, indent=1)
    d = O.make_desc(300, 37, 9)
    idx, w = O.conn_philox(d)
    sim = O.Sim(d, idx, w)
    sim.run(100)
    t, i = sim.raster()
    st = sim.state()
    rec = {"n": 300, "nsyn": 37, "seed": 9, "steps": 100, "tables_sha256": digest(idx, w),
           "raster_sha256": digest(t, i), "spikes": int(len(t)), "v_sha256": digest(st["v"]),
           "u_sha256": digest(st["u"])}
    with open(os.path.join(HERE, "oracle_small.json"), "w") as f:
        json.dump(rec, f, indent=1)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()

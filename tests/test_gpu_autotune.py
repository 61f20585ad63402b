"""Autotuning of contraction variants (itg_set_autotune / itg_autotune_*).

The reference caches one cuTENSOR algorithm per (mode, dim) key after timing
them all on first use (src/cudense.jl:284-326).  Here the variants are tile
shapes of the FP64 gather-GEMM (128x128, 128x64, 64x64), tile widths, CTA
clusters and stream-K scheduling of the split tcgen05 GEMM, and the tile of
grouped launches.  Every variant
must give bit-identical results, so tuning never changes an answer.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu


def _arr(t, xs):
    return (t * len(xs))(*xs)


def _shape_args(dA, mA, dB, mB, dC, mC):
    return (len(dA), _arr(C.c_int64, dA), _arr(C.c_int32, mA), len(dB), _arr(C.c_int64, dB), _arr(C.c_int32, mB),
            len(dC), _arr(C.c_int64, dC), _arr(C.c_int32, mC))


def _contract(h, a, dA, mA, b, dB, mB, dC, mC, prec=0):
    import torch
    out = torch.zeros(int(np.prod(dC)), dtype=torch.float64, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    h.call("itg_contract", 0, C.c_double(1.0), p(a), len(dA), _arr(C.c_int64, dA), _arr(C.c_int32, mA), p(b),
           len(dB), _arr(C.c_int64, dB), _arr(C.c_int32, mB), C.c_double(0.0), p(out), len(dC),
           _arr(C.c_int64, dC), _arr(C.c_int32, mC), prec)
    return out


CASES = [
    # (dims A, modes A, dims B, modes B, dims C, modes C): permuted, under-filling shapes
    ((40, 30, 50), (1, 2, 3), (50, 7, 30), (3, 4, 2), (7, 40), (4, 1)),
    ((300, 5, 260), (1, 2, 3), (260, 2, 2, 33), (3, 4, 5, 6), (33, 300, 2, 5, 2), (6, 1, 4, 2, 5)),
    ((129, 257), (1, 2), (257, 65), (2, 3), (129, 65), (1, 3)),
    # more output tiles than SMs: the stream-K variants share tiles between CTAs
    ((2560, 64), (1, 2), (64, 2048), (2, 3), (2560, 2048), (1, 3)),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_every_tile_variant_is_bit_identical(gpu, case):
    import torch
    from itg import _lib
    h = _lib.handle(0)
    dA, mA, dB, mB, dC, mC = CASES[case]
    rng = np.random.default_rng(case)
    A = rng.standard_normal(dA)
    B = rng.standard_normal(dB)
    a = torch.from_numpy(O.flat(A).copy()).cuda()
    b = torch.from_numpy(O.flat(B).copy()).cuda()
    outs = []
    for tile in (0, 1, 2):
        h.call("itg_autotune_force", *_shape_args(dA, mA, dB, mB, dC, mC), tile, 0)
        tq, bq = C.c_int(), C.c_int()
        h.call("itg_autotune_query", *_shape_args(dA, mA, dB, mB, dC, mC), C.byref(tq), C.byref(bq))
        assert tq.value == tile
        outs.append(_contract(h, a, dA, mA, b, dB, mB, dC, mC).cpu().numpy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    ref = O.contract(A, mA, B, mB, mC)
    got = O.unflat(outs[0], dC)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)
    # split: every tcgen05 variant gives identical bits too
    so = []
    # 256- / 128-wide tiles; 0x1000: stream-K
    for bn in (256, 128, 0x1000 | 256, 0x1000 | 128):
        h.call("itg_autotune_force", *_shape_args(dA, mA, dB, mB, dC, mC), -1, bn)
        so.append(_contract(h, a, dA, mA, b, dB, mB, dC, mC, prec=1).cpu().numpy())
    assert all(np.array_equal(so[0], x) for x in so[1:])
    refs = O.unflat(so[0], dC)
    assert np.linalg.norm(refs - ref) <= 1e-12 * np.linalg.norm(ref)
    h.call("itg_autotune_clear")


def test_autotune_runs_once_per_shape_and_caches(gpu):
    import torch
    from itg import _lib
    h = _lib.handle(0)
    h.call("itg_autotune_clear")
    h.call("itg_set_autotune", 1)
    e0, t0 = C.c_int64(), C.c_int64()
    h.call("itg_autotune_info", C.byref(e0), C.byref(t0))
    dA, mA, dB, mB, dC, mC = (96, 70, 80), (1, 2, 3), (80, 70, 24), (3, 2, 4), (96, 24), (1, 4)
    rng = np.random.default_rng(5)
    A, B = rng.standard_normal(dA), rng.standard_normal(dB)
    a = torch.from_numpy(O.flat(A).copy()).cuda()
    b = torch.from_numpy(O.flat(B).copy()).cuda()
    r1 = _contract(h, a, dA, mA, b, dB, mB, dC, mC).cpu().numpy()
    e1, t1 = C.c_int64(), C.c_int64()
    h.call("itg_autotune_info", C.byref(e1), C.byref(t1))
    assert t1.value == t0.value + 1 and e1.value == e0.value + 1
    r2 = _contract(h, a, dA, mA, b, dB, mB, dC, mC).cpu().numpy()
    e2, t2 = C.c_int64(), C.c_int64()
    h.call("itg_autotune_info", C.byref(e2), C.byref(t2))
    assert t2.value == t1.value and e2.value == e1.value
    assert np.array_equal(r1, r2)
    ref = O.contract(A, mA, B, mB, mC)
    assert np.linalg.norm(O.unflat(r1, dC) - ref) <= 1e-12 * np.linalg.norm(ref)
    # tuning off: no new tuning for a new shape
    h.call("itg_set_autotune", 0)
    dA2 = (97, 70, 80)
    a2 = torch.from_numpy(O.flat(rng.standard_normal(dA2)).copy()).cuda()
    _contract(h, a2, dA2, mA, b, dB, mB, (97, 24), mC)
    e3, t3 = C.c_int64(), C.c_int64()
    h.call("itg_autotune_info", C.byref(e3), C.byref(t3))
    assert t3.value == t2.value
    h.call("itg_set_autotune", 1)
    h.call("itg_autotune_clear")


def test_autotune_file_round_trip(gpu, tmp_path):
    """ITG_TUNE_FILE: choices are appended as 'key value' lines and read back
    by a fresh process."""
    import subprocess
    import sys
    import textwrap
    f = tmp_path / "tune.txt"
    code = textwrap.dedent("""
        import ctypes as C, sys
        sys.path[:0] = sys.argv[1:3]
        import numpy as np, torch
        from itg import _lib
        h = _lib.handle(0)
        arr = lambda t, xs: (t * len(xs))(*xs)
        a = torch.randn(60 * 50, dtype=torch.float64, device="cuda")
        b = torch.randn(50 * 40, dtype=torch.float64, device="cuda")
        c = torch.zeros(60 * 40, dtype=torch.float64, device="cuda")
        p = lambda t: C.c_void_p(t.data_ptr())
        h.call("itg_contract", 0, C.c_double(1.0), p(a), 2, arr(C.c_int64, [60, 50]), arr(C.c_int32, [1, 2]),
               p(b), 2, arr(C.c_int64, [50, 40]), arr(C.c_int32, [2, 3]), C.c_double(0.0), p(c), 2,
               arr(C.c_int64, [60, 40]), arr(C.c_int32, [1, 3]), 0)
        e, t = C.c_int64(), C.c_int64()
        h.call("itg_autotune_info", C.byref(e), C.byref(t))
        print(e.value, t.value)
    """)
    from pathlib import Path
    repo = Path(__file__).resolve().parent.parent
    env = dict(__import__("os").environ, ITG_TUNE_FILE=str(f), ITG_AUTOTUNE="1")
    args = [sys.executable, "-c", code, str(repo), str(repo / "itensorsgpu.jl_gb300")]
    out1 = subprocess.run(args, env=env, capture_output=True, text=True, timeout=300)
    assert out1.returncode == 0, out1.stderr
    assert out1.stdout.split() == ["1", "1"]
    lines = f.read_text().strip().splitlines()
    assert len(lines) == 1 and lines[0].startswith("f64|")
    out2 = subprocess.run(args, env=env, capture_output=True, text=True, timeout=300)
    assert out2.returncode == 0, out2.stderr
    assert out2.stdout.split() == ["1", "0"]  # read from the file, not re-tuned


def test_grouped_tuned_equals_single(gpu):
    """Grouped launches under every tile choice equal the single contractions."""
    import torch
    from itg import _lib
    h = _lib.handle(0)
    h.call("itg_autotune_clear")
    rng = np.random.default_rng(8)
    dims = [(17, 33, 9), (40, 12, 31), (64, 64, 64), (5, 100, 7)]
    As, Bs, Cs, refs = [], [], [], []
    for m, k, n in dims:
        A = rng.standard_normal((m, k))
        B = rng.standard_normal((k, n))
        As.append(torch.from_numpy(O.flat(A).copy()).cuda())
        Bs.append(torch.from_numpy(O.flat(B).copy()).cuda())
        Cs.append(torch.zeros(m * n, dtype=torch.float64, device="cuda"))
        refs.append(A @ B)
    ptrs = lambda ts: (C.c_void_p * len(ts))(*[C.c_void_p(t.data_ptr()) for t in ts])
    flat = lambda f: [x for d in dims for x in f(*d)]
    for rep in range(2):  # first call tunes, second uses the cache
        for c in Cs:
            c.zero_()
        h.call("itg_contract_grouped", len(dims), C.c_double(1.0), ptrs(As), 2,
               _arr(C.c_int64, flat(lambda m, k, n: (m, k))), _arr(C.c_int32, [1, 2]), ptrs(Bs), 2,
               _arr(C.c_int64, flat(lambda m, k, n: (k, n))), _arr(C.c_int32, [2, 3]), C.c_double(0.0), ptrs(Cs), 2,
               _arr(C.c_int64, flat(lambda m, k, n: (m, n))), _arr(C.c_int32, [1, 3]))
        for c, r, (m, k, n) in zip(Cs, refs, dims):
            got = O.unflat(c.cpu().numpy(), (m, n))
            assert np.linalg.norm(got - r) <= 1e-12 * np.linalg.norm(r)
    h.call("itg_autotune_clear")

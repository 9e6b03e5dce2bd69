"""GPU parity of the stencil time loop (2D and 3D) through the C ABI.

Reference evaluation order must be bit-identical to the reference's CPU gold
code (golden fixtures) and to the oracle on ragged sizes, for both kernels
(persistent with resident rows/planes, and one launch per step), both sweep
modes and both boundary modes. The fast (FMA) order is checked against the
oracle with tolerances stated below."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPES2D = ["2d5pt", "2ds9pt", "2d13pt", "2d17pt", "2d21pt", "2ds25pt", "2d9pt", "2d25pt"]
SHAPES3D = ["3d7pt", "3d13pt", "3d17pt", "3d27pt", "poisson"]


def bits_equal(a, b):
    """Bit-identical, except that any NaN equals any NaN (x86 and the GPU
    produce different NaN payloads for the same invalid operation)."""
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    return np.array_equal(a[~na].view(np.uint8), b[~nb].view(np.uint8))


def run(native, cuda, field, shape, steps, **kw):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(field)).to(cuda)
    if field.ndim == 2:
        out, st = native.stencil2d(t, shape, steps, **kw)
    else:
        out, st = native.stencil3d(t, shape, steps, **kw)
    torch.cuda.synchronize()
    return out.cpu().numpy(), st


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(HERE, "golden", "stencil_golden.npz"))


@pytest.mark.parametrize("shape", SHAPES2D + SHAPES3D)
@pytest.mark.parametrize("dt", ["float32", "float64"])
@pytest.mark.parametrize("kernel", ["persistent", "per_step"])
def test_golden_bit_exact(native, cuda, golden, shape, dt, kernel):
    f = golden[f"{shape}_{dt}_in"]
    for s in (1, 2, 7):
        g, _ = run(native, cuda, f, shape, s, kernel=kernel)
        assert bits_equal(g, golden[f"{shape}_{dt}_s{s}"]), (shape, dt, kernel, s)


CASES_2D = [
    # (wy, wx, ctas, steps)  — ragged, multi-column-tile, tall tiles with many resident rows
    ((1, 1), 0, 3), ((1, 37), 0, 2), ((37, 1), 0, 2), ((13, 1030), 0, 5), ((300, 2100), 0, 4),
    ((2000, 700), 0, 7), ((1500, 1100), 6, 9), ((777, 3000), 9, 6),
]


@pytest.mark.parametrize("shape", SHAPES2D)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_2d_ragged_vs_oracle(native, cuda, oracle, shape, dt):
    rng = np.random.default_rng(11)
    for (dims, ctas, steps) in CASES_2D:
        f = rng.random(dims).astype(dt)
        ref = oracle.stencil(shape, f, steps)
        for kw in ({"kernel": "persistent", "ctas": ctas}, {"kernel": "per_step", "ctas": ctas},
                   {"kernel": "persistent", "ctas": ctas, "l2_sweep": True},
                   {"kernel": "persistent", "ctas": ctas, "cache_rows": 0}, {"kernel": "naive"}):
            g, st = run(native, cuda, f, shape, steps, **kw)
            assert bits_equal(g, ref), (shape, dims, kw, steps, np.nanmax(np.abs(g - ref)))


def test_2d_resident_rows_are_used(native, cuda, oracle):
    f = np.random.default_rng(3).random((1500, 1100))
    g, st = run(native, cuda, f, "2d5pt", 9, ctas=6)
    assert st["cached_rows"] > 0 and st["cached_fraction"] > 0
    assert bits_equal(g, oracle.stencil("2d5pt", f, 9))


CASES_3D = [((1, 1, 1), 0, 2), ((3, 5, 7), 0, 3), ((17, 33, 70), 0, 4), ((40, 70, 130), 4, 5),
            ((64, 40, 66), 2, 6), ((9, 100, 200), 0, 3),
            # widths one or two columns past a tile edge (64/128/256-column tiles)
            ((6, 40, 257), 5, 3), ((4, 33, 129), 3, 3), ((4, 20, 65), 2, 4), ((3, 9, 258), 0, 3)]


@pytest.mark.parametrize("shape", SHAPES3D)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_3d_ragged_vs_oracle(native, cuda, oracle, shape, dt):
    rng = np.random.default_rng(12)
    for (dims, ctas, steps) in CASES_3D:
        f = rng.random(dims).astype(dt)
        ref = oracle.stencil(shape, f, steps)
        for kw in ({"kernel": "persistent", "ctas": ctas}, {"kernel": "per_step"},
                   {"kernel": "persistent", "ctas": ctas, "l2_sweep": True}):
            g, st = run(native, cuda, f, shape, steps, **kw)
            assert bits_equal(g, ref), (shape, dims, kw, steps, np.nanmax(np.abs(g - ref)))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape", ["3d7pt", "3d13pt", "3d27pt"])
def test_3d_work_split(native, cuda, oracle, dt, shape):
    # Every CTA takes an equal run of (tile, plane) pairs: runs that start and
    # end inside tiles, span two tiles, or are shorter than the stencil's reach.
    f = np.random.default_rng(4).random((37, 70, 300)).astype(dt)
    ref = oracle.stencil(shape, f, 4)
    for ctas in (1, 3, 7, 13, 50, 152):
        for l2 in (False, True):
            g, st = run(native, cuda, f, shape, 4, ctas=ctas, l2_sweep=l2)
            assert bits_equal(g, ref), (shape, dt, ctas, l2)


@pytest.mark.parametrize("shape", ["2d5pt", "2ds25pt", "2d25pt", "3d7pt", "3d27pt", "poisson"])
@pytest.mark.parametrize("kernel", ["persistent", "per_step", "naive"])
def test_dirichlet_vs_oracle(native, cuda, oracle, shape, kernel):
    if kernel == "naive" and not shape.startswith("2d"):
        pytest.skip("the naive comparator is 2D only, as in the reference")
    dims = (300, 517) if shape.startswith("2d") else (20, 37, 70)
    f = np.random.default_rng(5).random(dims)
    g, _ = run(native, cuda, f, shape, 5, kernel=kernel, boundary="dirichlet")
    assert bits_equal(g, oracle.stencil(shape, f, 5, boundary=1))


# Fast (FMA, folded coefficient) order. Tolerance: per-cell relative error
# vs the FP64 reference-order oracle, 1e-12 for FP64 (the plain FP64 path's per-cell bound),
# 2e-5 for FP32 storage; shapes with positive weights only, so values stay
# away from zero and the relative error is meaningful.
@pytest.mark.parametrize("shape", ["2d5pt", "2ds9pt", "2ds25pt", "2d9pt", "2d25pt", "3d27pt", "3d17pt"])
@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-12), (np.float32, 2e-5)])
def test_fast_order_within_tolerance(native, cuda, oracle, shape, dt, tol):
    dims = (400, 1300) if shape.startswith("2d") else (30, 45, 80)
    f = np.random.default_rng(6).random(dims)
    ref = oracle.stencil(shape, f, 20)
    g, _ = run(native, cuda, f.astype(dt), shape, 20, order="fast")
    rel = np.abs(g.astype(np.float64) - ref) / np.abs(ref)
    assert rel.max() <= tol, rel.max()


def test_zero_steps_copies(native, cuda):
    f = np.random.default_rng(7).random((33, 65))
    g, _ = run(native, cuda, f, "2d5pt", 0)
    assert bits_equal(g, f)


def test_large_field_properties(native, cuda, oracle):
    """Full-size 2D field (8192^2 FP32): persistent == per-step bit for bit,
    and a 64-row band well inside the domain agrees with the oracle run on a
    crop wide enough that the crop's edges cannot reach it."""
    import torch
    wy = wx = 8192
    steps = 6
    g = torch.Generator(device="cpu").manual_seed(1)
    f = torch.rand((wy, wx), generator=g, dtype=torch.float32)
    d = f.to(cuda)
    a, _ = native.stencil2d(d, "2ds9pt", steps, kernel="persistent", l2_sweep=True)
    b, _ = native.stencil2d(d, "2ds9pt", steps, kernel="per_step")
    assert torch.equal(a, b)
    H = 2 * steps
    y0, x0, n = 4000, 3000, 64
    crop = f[y0 - H:y0 + n + H, x0 - H:x0 + n + H].numpy()
    ref = oracle.stencil("2ds9pt", crop, steps)[H:H + n, H:H + n]
    assert bits_equal(a[y0:y0 + n, x0:x0 + n].cpu().numpy(), ref)


@pytest.mark.parametrize("shape", ["2d5pt", "2ds9pt", "2d13pt", "2d21pt", "2ds25pt", "2d9pt", "2d25pt", "3d17pt",
                                   "3d27pt", "3d7pt"])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_extreme_values_bit_exact(native, cuda, oracle, shape, dt):
    """Subnormal, tiny, huge, infinite and NaN inputs: exercises the exact
    constant-division paths against the reference order on the CPU, in
    every finish form the FP32 star shapes use (2d5pt full, 2d21pt the
    warp-vote short path, the others the branch-free short finish)."""
    rng = np.random.default_rng(21)
    dims = (64, 200) if shape.startswith("2d") else (12, 20, 70)
    tiny = np.finfo(dt).smallest_subnormal
    big = np.finfo(dt).max
    f = rng.random(dims)
    scale = rng.choice(np.array([tiny * 7, tiny * 1e3, np.finfo(dt).tiny, 1e-3, 1.0, big / 200, big / 20],
                                dtype=np.float64), size=dims)
    f = (f * scale).astype(dt)
    flat = f.reshape(-1)
    flat[::97] = np.inf
    flat[5::131] = -0.0
    flat[7::173] = np.nan
    flat[11::59] = -flat[11::59]
    for s in (1, 3):
        g, _ = run(native, cuda, f, shape, s)
        assert bits_equal(g, oracle.stencil(shape, f, s)), (shape, dt, s)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_decay_through_subnormals(native, cuda, oracle, dt):
    """2d5pt decays to zero through the subnormal range (FP32 in ~80 steps,
    FP64 in ~800): every step must stay bit-identical."""
    f = np.random.default_rng(22).random((96, 160)).astype(dt)
    steps = 140 if dt == np.float32 else 900
    g, _ = run(native, cuda, f, "2d5pt", steps)
    assert bits_equal(g, oracle.stencil("2d5pt", f, steps))


@pytest.mark.parametrize("shape,dt,dims", [("2d5pt", np.float32, (300, 517)), ("2ds9pt", np.float32, (64, 8192)),
                                           ("2d25pt", np.float64, (77, 1000)), ("3d7pt", np.float32, (20, 33, 70)),
                                           ("3d27pt", np.float64, (9, 40, 130)), ("poisson", np.float32, (5, 6, 7))])
def test_host_buffer_dropins(native, cuda, oracle, shape, dt, dims):
    """jacobi_iterative / j3d_iterative: host arrays (pageable and pinned) in
    and out, copied straight to and from the internal fields."""
    import torch
    f = np.random.default_rng(21).random(dims).astype(dt)
    ref = oracle.stencil(shape, f, 6)
    pinned_in = torch.from_numpy(f.copy()).pin_memory().numpy()
    pinned_out = torch.empty(dims, dtype=torch.from_numpy(f).dtype).pin_memory().numpy()
    for src, dst in ((f, np.empty_like(f)), (pinned_in, pinned_out)):
        for warm in (False, True):
            dst[...] = np.nan
            if len(dims) == 2:
                rc = native.jacobi_iterative(src, dims[0], dims[1], dst, iteration=6, usewarmup=warm,
                                             warmupiteration=2, shape=shape)
            else:
                rc = native.j3d_iterative(src, dims[0], dims[1], dims[2], dst, iteration=6, usewarmup=warm,
                                          warmupiteration=2, shape=shape)
            assert rc == 0, native.last_error()
            assert bits_equal(dst, ref), (shape, warm)
    # zero steps copies
    dst = np.empty_like(f)
    if len(dims) == 2:
        assert native.jacobi_iterative(f, dims[0], dims[1], dst, iteration=0, shape=shape) == 0
    else:
        assert native.j3d_iterative(f, dims[0], dims[1], dims[2], dst, iteration=0, shape=shape) == 0
    assert bits_equal(dst, f)

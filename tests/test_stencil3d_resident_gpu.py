"""3D resident planes (PERKS caching in the 3D kernel): plane tiles of a
CTA's z-run that no other CTA reads stay in shared memory for the whole
persistent launch. The kernel copies them into its ring by shared-to-shared
bulk copies and writes to the field only the rows and columns that the
neighbouring tiles read. Small grids (few CTAs, long z-runs) make every
shape keep planes; every result must stay bit-identical to the oracle and to
the same run without resident planes, for both sweep modes and both
boundaries, and at the minimum domain height, where every CTA keeps every
plane that no other CTA reads."""
import numpy as np
import pytest

from test_stencil_gpu import SHAPES3D, bits_equal, run

pytestmark = pytest.mark.gpu

CASES = [((40, 70, 130), 4, 5), ((64, 40, 66), 2, 6), ((33, 33, 257), 3, 4), ((50, 9, 40), 1, 7),
         ((21, 100, 129), 5, 3)]


@pytest.mark.parametrize("shape", SHAPES3D)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("order", ["reference", "fast"])
def test_resident_planes_vs_oracle(native, cuda, oracle, shape, dt, order):
    """Where the tuned tile leaves no room for a plane next to its ring
    (FP32 3d13pt both orders, FP32 fast 3d7pt) nothing is kept; elsewhere
    planes are. Reference order: bit-identical to the oracle; fast order:
    bit-identical with and without resident planes and in both sweep modes."""
    from perks_gb300.stencil import min_domain_3d
    fits = min_domain_3d(shape, 64, 64, dt, order=order, cache_rows=-1) > 0
    rng = np.random.default_rng(41)
    for dims, ctas, steps in CASES:
        f = rng.random(dims).astype(dt)
        ref = oracle.stencil(shape, f, steps)
        base = None
        for kw in ({"cache_rows": -1}, {"cache_rows": -1, "l2_sweep": True}, {"cache_rows": 1}, {"cache_rows": 0},
                   {}):
            g, st = run(native, cuda, f, shape, steps, kernel="persistent", ctas=ctas, order=order, **kw)
            cached = kw.get("cache_rows", 0) != 0 and fits  # the 3D default keeps none
            assert (st["cached_rows"] > 0) == cached and (st["cached_fraction"] > 0) == cached, (shape, dims, st)
            if order == "reference":
                assert bits_equal(g, ref), (shape, dt, dims, ctas, kw)
            else:
                # the same arithmetic with and without resident planes
                base = g if base is None else base
                assert bits_equal(g, base), (shape, dt, dims, ctas, kw)


@pytest.mark.parametrize("shape", ["3d7pt", "3d27pt", "poisson"])
def test_resident_planes_dirichlet(native, cuda, oracle, shape):
    f = np.random.default_rng(42).random((40, 50, 70))
    ref = oracle.stencil(shape, f, 6, boundary=1)
    g, st = run(native, cuda, f, shape, 6, kernel="persistent", ctas=3, boundary="dirichlet", cache_rows=-1)
    assert st["cached_rows"] > 0
    assert bits_equal(g, ref)


def _split(h, tiles, grid, H, kr):
    """The kernel's split of the (tile, plane) pairs over `grid` CTAs, and per
    CTA its planes off the z-run ends (H at each end) and the resident ones."""
    total = tiles * h
    grid = min(grid, total)
    out = []
    for b in range(grid):
        c_lo, c_hi = total * b // grid, total * (b + 1) // grid
        inner, best = 0, 0
        for tb in range(c_lo // h, (c_hi - 1) // h + 1):
            zl, zh = max(c_lo, tb * h) - tb * h, min(c_hi, (tb + 1) * h) - tb * h
            n = max(0, (zh - H) - (zl + H))
            inner += n
            best = max(best, min(kr, n))
        out.append((inner, best))
    return total, out


@pytest.mark.parametrize("shape,dt", [("3d7pt", np.float32), ("3d13pt", np.float64), ("3d27pt", np.float32),
                                      ("3d17pt", np.float64)])
def test_min_domain_height(native, cuda, oracle, shape, dt):
    """At the minimum-domain height every plane of every CTA's z-runs but the
    H at each end is resident; the reported cached fraction is exactly that
    share of the (tile, plane) pairs, and one plane higher no longer fits."""
    import torch
    from perks_gb300.stencil import min_domain_3d
    wy = wx = 256
    h = min_domain_3d(shape, wy, wx, dt, cache_rows=-1)
    assert h > 0
    # the reference-signature query (getminHeight = 1, useSM = 1) gives the same height
    L = native.lib()
    query = L.perks_j3d_iterative_f64 if dt == np.float64 else L.perks_j3d_iterative_f32
    assert query(native.SHAPES[shape], None, 0, wy, wx, None, 256, 0, 0, 1, 0, 0, 0, 1) == h
    f = np.random.default_rng(43).random((h, wy, wx)).astype(dt)
    g, st = run(native, cuda, f, shape, 4, kernel="persistent", cache_rows=-1)
    assert bits_equal(g, oracle.stencil(shape, f, 4))
    H = native.HALO[shape]
    sms = torch.cuda.get_device_properties(cuda).multi_processor_count
    tiles = st["grid_x"] * st["grid_y"]
    total, per_cta = _split(h, tiles, sms, H, st["cached_rows"])
    assert all(inner == best for inner, best in per_cta), per_cta
    assert st["cached_fraction"] == pytest.approx(sum(b for _, b in per_cta) / total, abs=1e-12)
    assert st["cached_fraction"] > 0
    _, above = _split(h + 1, tiles, sms, H, st["cached_rows"])
    assert not all(inner == best for inner, best in above)
    assert min_domain_3d(shape, wy, wx, dt, cache_rows=0) == 0
    assert min_domain_3d(shape, wy, wx, dt) == 0  # the 3D default keeps no planes

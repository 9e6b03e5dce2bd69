"""The TMA-fed 2D kernel (perks_stencil_opts.tma = 1): rows reach each warp's
shared-memory ring by cp.async.bulk.tensor.2d copies issued by one lane and
completed on a per-slot mbarrier, instead of per-lane cp.async. Same
arithmetic, so every result must be bit-identical to the oracle (reference
order) on the golden fixtures and on ragged sizes (single columns and rows,
widths one past a strip, strips of 128/256 columns, resident rows on and
off, both sweep modes, both boundaries), and bit-identical to the cp.async
kernel on a full 8192^2 field."""
import numpy as np
import pytest

from test_stencil_gpu import CASES_2D, SHAPES2D, bits_equal, golden, run  # noqa: F401 (golden: fixture)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", SHAPES2D)
@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_tma_golden_bit_exact(native, cuda, golden, shape, dt):
    f = golden[f"{shape}_{dt}_in"]
    for kernel in ("persistent", "per_step"):
        for s in (1, 2, 7):
            g, _ = run(native, cuda, f, shape, s, kernel=kernel, tma=True)
            assert bits_equal(g, golden[f"{shape}_{dt}_s{s}"]), (shape, dt, kernel, s)


EXTRA = [((5, 129), 0, 3), ((40, 257), 2, 4), ((64, 256), 1, 5), ((33, 513), 3, 4), ((9, 65), 0, 6)]


@pytest.mark.parametrize("shape", SHAPES2D)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_tma_ragged_vs_oracle(native, cuda, oracle, shape, dt):
    rng = np.random.default_rng(13)
    for (dims, ctas, steps) in CASES_2D + EXTRA:
        f = rng.random(dims).astype(dt)
        ref = oracle.stencil(shape, f, steps)
        for kw in ({"kernel": "persistent", "ctas": ctas}, {"kernel": "per_step", "ctas": ctas},
                   {"kernel": "persistent", "ctas": ctas, "l2_sweep": True},
                   {"kernel": "persistent", "ctas": ctas, "cache_rows": 0}):
            g, st = run(native, cuda, f, shape, steps, tma=True, **kw)
            assert bits_equal(g, ref), (shape, dims, kw, steps, np.nanmax(np.abs(g - ref)))


@pytest.mark.parametrize("shape", ["2d5pt", "2ds25pt", "2d25pt"])
def test_tma_dirichlet_vs_oracle(native, cuda, oracle, shape):
    f = np.random.default_rng(14).random((300, 517))
    ref = oracle.stencil(shape, f, 5, boundary=1)
    for kernel in ("persistent", "per_step"):
        g, _ = run(native, cuda, f, shape, 5, kernel=kernel, boundary="dirichlet", tma=True)
        assert bits_equal(g, ref), (shape, kernel)


def test_tma_resident_rows_are_used(native, cuda, oracle):
    f = np.random.default_rng(3).random((1500, 1100)).astype(np.float32)
    g, st = run(native, cuda, f, "2ds9pt", 9, ctas=6, tma=True)
    assert st["cached_rows"] > 0 and st["cached_fraction"] > 0
    assert bits_equal(g, oracle.stencil("2ds9pt", f, 9))


def test_tma_matches_cp_async_full_field(native, cuda):
    import torch
    g = torch.Generator(device="cpu").manual_seed(2)
    d = torch.rand((8192, 8192), generator=g, dtype=torch.float32).to(cuda)
    for kw in ({"kernel": "persistent"}, {"kernel": "persistent", "l2_sweep": True}, {"kernel": "per_step"}):
        a, _ = native.stencil2d(d, "2ds9pt", 6, **kw)
        b, _ = native.stencil2d(d, "2ds9pt", 6, tma=True, **kw)
        assert torch.equal(a, b), kw
        del a, b

"""Minimum-domain mode (the reference's --small: getMinWidthY,
stencil/2dstencil/jacobi-2d.cu:79-136, used by jacobi.driver.cpp:84-109).

At the width_y the query returns, the persistent kernel must keep every row
of every band on chip except the H rows at each end of the band, and the
results must stay bit-identical to the oracle; one more row per band must no
longer fit."""
import numpy as np
import pytest

from test_stencil_gpu import bits_equal, run

pytestmark = pytest.mark.gpu

CASES = [("2d5pt", np.float32, 1024, 0), ("2ds9pt", np.float32, 3000, 0), ("2d13pt", np.float32, 700, 7),
         ("2ds25pt", np.float32, 2100, 0), ("2d9pt", np.float64, 1024, 0), ("2d25pt", np.float32, 900, 5),
         ("2d21pt", np.float64, 1500, 0), ("2d5pt", np.float64, 100, 3)]


@pytest.mark.parametrize("shape,dt,wx,ctas", CASES)
def test_min_domain_is_fully_cached(native, cuda, oracle, shape, dt, wx, ctas):
    H = native.HALO[shape]
    wy = native.min_domain_2d(shape, wx, dt, ctas=ctas)
    assert wy > 0
    rng = np.random.default_rng(wy)
    f = rng.random((wy, wx)).astype(dt)
    g, st = run(native, cuda, f, shape, 3, ctas=ctas)
    nb = st["grid_y"]
    assert wy % nb == 0 and st["cached_rows"] == wy // nb - 2 * H
    assert abs(st["cached_fraction"] * wy - (wy - 2 * H * nb)) < 0.5
    assert bits_equal(g, oracle.stencil(shape, f, 3))
    # one more row in every band: the band's interior no longer fits
    f2 = rng.random((wy + nb, wx)).astype(dt)
    g2, st2 = run(native, cuda, f2, shape, 2, ctas=ctas)
    assert st2["grid_y"] == nb and st2["cached_rows"] == st["cached_rows"]
    assert st2["cached_fraction"] * (wy + nb) < (wy + nb) - 2 * H * nb - 0.5
    assert bits_equal(g2, oracle.stencil(shape, f2, 2))


def test_min_domain_without_cache(native, cuda):
    assert native.min_domain_2d("2d5pt", 1024, kernel="per_step") == 0
    assert native.min_domain_2d("2d5pt", 1024, cache_rows=0) == 0
    assert native.getMinWidthY(1024, useSM=False, shape="2d5pt") == 0
    # the reference-signature query agrees with the options form
    assert native.getMinWidthY(1024, shape="2ds9pt") == native.min_domain_2d("2ds9pt", 1024)
    assert native.getMinWidthY(1024, shape="2d9pt", dtype=np.float64) == \
        native.min_domain_2d("2d9pt", 1024, np.float64)
    # a smaller cache_rows limit gives a proportionally smaller domain
    full = native.min_domain_2d("2d5pt", 1024)
    two = native.min_domain_2d("2d5pt", 1024, cache_rows=2)
    assert 0 < two < full and two % (2 + 2 * native.HALO["2d5pt"]) == 0


def test_j3d_min_height(native, cuda):
    """getminHeight answers the 3D minimum-domain height (resident plane
    tiles), and 0 without shared-memory caching (the reference's no-cache
    answer)."""
    h = native.j3d_iterative(None, 64, 64, 64, None, getminHeight=True, shape="3d7pt")
    assert h > 0 and h == native.min_domain_3d("3d7pt", 64, 64, cache_rows=-1)
    assert native.j3d_iterative(None, 64, 64, 64, None, getminHeight=True, useSM=False, shape="3d7pt") == 0


def test_min_domain_rejects_too_wide(native, cuda):
    with pytest.raises(native.PerksError):
        native.min_domain_2d("2d5pt", 1 << 30)

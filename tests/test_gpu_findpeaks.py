"""Peak search on a caller's grid (fo_findpeaks, the Fortran FINDPEAKS)
against the oracle: the 5^3-window kernel, the wider-window kernel (start
half-widths 1 and 3), mixed precision and the no-peak stop."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gaussian_grid(n, seed, npk=4):
    """Periodic n^3 grid [i1, i2, i3]: a few anisotropic Gaussians of distinct
    heights on a constant background."""
    rng = np.random.default_rng(seed)
    idx = np.indices((n, n, n)).astype(float)
    f = np.full((n, n, n), 0.3)
    for k in range(npk):
        c = rng.uniform(0, n, 3)
        w = rng.uniform(1.0, 2.2, 3)
        d2 = 0.0
        for a in range(3):
            d = idx[a] - c[a]
            d -= n * np.round(d / n)
            d2 = d2 + (d / w[a]) ** 2
        f += (3.0 - 0.6 * k) * np.exp(-d2)
    return f


@pytest.mark.parametrize("n", [12, 16, 24])
@pytest.mark.parametrize("width", [1, 2, 3])
def test_findpeaks_fp64_matches_oracle(fo, oracle_mod, n, width):
    f = gaussian_grid(n, seed=n + 7 * width)
    pk_o, am_o = oracle_mod.findpeaks(f, 6, width=width)
    pk, am = fo.findpeaks(f, 6, width=width, precision="fp64")
    assert pk.shape == pk_o.shape
    np.testing.assert_allclose(pk, pk_o, rtol=0, atol=1e-5)
    np.testing.assert_allclose(am, am_o, rtol=1e-5, atol=1e-7)


def test_findpeaks_mixed_close_to_oracle(fo, oracle_mod):
    f = gaussian_grid(16, seed=3)
    pk_o, am_o = oracle_mod.findpeaks(f, 4)
    pk, am = fo.findpeaks(f, 4, precision="mixed")
    assert pk.shape == pk_o.shape
    # FP32 grid and fit (tolerance 1e-5): centres within a few thousandths of a cell
    np.testing.assert_allclose(pk, pk_o, rtol=0, atol=5e-3)
    np.testing.assert_allclose(am, am_o, rtol=5e-3)


def test_findpeaks_no_peak_stops(fo, oracle_mod):
    f = gaussian_grid(12, seed=5)
    f[0, 0, 0] = np.nan          # every fit starts from a non-finite cost
    with pytest.raises(RuntimeError):
        oracle_mod.findpeaks(f, 3)
    with pytest.raises(fo.FoError) as e:
        fo.findpeaks(f, 3, precision="fp64")
    assert e.value.status == 2


def test_findpeaks_argument_errors(fo):
    f = gaussian_grid(8, seed=1)
    for kw in ({"width": 0}, {"width": 8}, {"npeaks": 0}, {"npeaks": 65}):
        args = {"npeaks": 3, **kw}
        with pytest.raises(fo.FoError):
            fo.findpeaks(f, args.pop("npeaks"), **args)
    with pytest.raises(ValueError):
        fo.findpeaks(np.zeros((4, 4, 5)), 2)

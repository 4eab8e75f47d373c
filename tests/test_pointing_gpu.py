"""Pointing -> pixel index on the GPU (mk_pix_car, mk_pix_wcs_car) against
the reference's own outputs (pointing.npz) and the oracle.  GPU only."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda", 0)


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    return t.to(dtype) if dtype is not None else t


@pytest.fixture(scope="module")
def K():
    from minkasi_gb300 import kernels
    return kernels


def test_pix_car_bit_exact_with_reference(K, gold):
    g = gold("pointing.npz")
    for k in range(int(g["ncase"])):
        ra, dec, lims = dev(g[f"c{k}_ra"]), dev(g[f"c{k}_dec"]), g[f"c{k}_lims"]
        ps, ny, cosdec = float(g[f"c{k}_pixsize"]), int(g[f"c{k}_ny"]), float(g[f"c{k}_cosdec"])
        car = K.pix_car(ra, dec, lims[0], lims[2], ps, cosdec, ny, trunc=False)
        assert np.array_equal(car.cpu().numpy(), g[f"c{k}_car"]), k
        tr = K.pix_car(ra, dec, lims[0], lims[2], ps, cosdec, ny, trunc=True)
        assert np.array_equal(tr.cpu().numpy(), g[f"c{k}_trunc"]), k


def test_skymapcar_get_pix_and_radec2pix_car(gold):
    import minkasi_gb300 as mk
    g = gold("pointing.npz")
    for k in range(int(g["ncase"])):
        lims, ps, ny = list(g[f"c{k}_lims"]), float(g[f"c{k}_pixsize"]), int(g[f"c{k}_ny"])
        m = mk.SkyMapCar(lims, ps, nx=ny, ny=ny)
        tod = mk.Tod({"dx": g[f"c{k}_ra"], "dy": g[f"c{k}_dec"],
                      "dat_calib": np.zeros(g[f"c{k}_ra"].shape)})
        ipix = m.pix_from_radec(tod.info["dx"], tod.info["dy"])
        assert np.array_equal(ipix.cpu().numpy(), g[f"c{k}_car"])
        out = torch.empty(g[f"c{k}_ra"].shape, dtype=torch.int32, device=cuda)
        mk.radec2pix_car(g[f"c{k}_ra"], g[f"c{k}_dec"], out, lims, ps, float(g[f"c{k}_cosdec"]), ny)
        assert np.array_equal(out.cpu().numpy(), g[f"c{k}_trunc"])


@pytest.mark.parametrize("ref_equ", [False, True])
@pytest.mark.parametrize("centre", [(3.5, 0.31), (0.7, -0.42), (1.2, 0.0)])
def test_pix_wcs_car_matches_oracle(K, centre, ref_equ):
    """The CAR WCS kernel against the oracle's restatement of the same
    equations (parity with astropy is unpinned: astropy is absent)."""
    rng = np.random.default_rng(int(centre[0] * 10) + int(ref_equ))
    arcsec = np.pi / 180 / 3600
    half = 900 * arcsec
    ra_c, dec_c = centre
    lims = [ra_c - half, ra_c + half, dec_c - half, dec_c + half]
    ps = 1.5 * arcsec
    w = oracle.car_wcs(lims, ps, ref_equ)
    ra = ra_c + rng.uniform(-1, 1, size=200_000) * half
    dec = dec_c + rng.uniform(-1, 1, size=200_000) * half
    ny = 1300
    ref = oracle.pix_wcs_car(ra, dec, w, ny)
    got = K.pix_wcs_car(dev(ra), dev(dec), w, ny).cpu().numpy()
    assert np.array_equal(got, ref)


def test_skymap_wcs_size_and_get_pix_caches(K):
    import minkasi_gb300 as mk
    arcsec = np.pi / 180 / 3600
    lims = [3.5 - 0.01, 3.5 + 0.01, 0.3 - 0.008, 0.3 + 0.008]
    ps = 2 * arcsec
    m = mk.SkyMap(lims, ps)
    w = oracle.car_wcs(lims, ps)
    corners = [oracle.wcs_car_world2pix(np.array([lims[a] * 180 / np.pi]), np.array([lims[b] * 180 / np.pi]), w)
               for a, b in ((0, 2), (0, 3), (1, 2), (1, 3))]
    nx = int(max(np.round(c[0][0]) for c in corners) + 2)
    ny = int(max(np.round(c[1][0]) for c in corners) + 2)
    assert (m.nx, m.ny) == (nx, ny)
    rng = np.random.default_rng(4)
    ra = rng.uniform(lims[0], lims[1], size=(4, 5000))
    dec = rng.uniform(lims[2], lims[3], size=(4, 5000))
    tod = mk.Tod({"dx": ra, "dy": dec, "dat_calib": np.ones((4, 5000))})
    ipix = m.get_pix(tod)
    assert np.array_equal(ipix.cpu().numpy(), oracle.pix_wcs_car(ra, dec, np.asarray(w), m.ny))
    assert "ipix" in tod.info  # cached under the map's tag, as the reference does
    m.tod2map(tod, tod.info["dat_calib"])
    assert float(m.map.sum().item()) == 4 * 5000


def test_pix_nan_and_empty(K):
    ra = dev(np.array([np.nan, 0.1, 1e30]))
    dec = dev(np.array([0.0, 0.0, 0.0]))
    out = K.pix_car(ra, dec, 0.0, 0.0, 1e-3, 1.0, 100).cpu().numpy()
    assert out[0] == np.iinfo(np.int32).min and out[2] == np.iinfo(np.int32).min
    assert out[1] == np.asarray(np.round(0.1 / 1e-3) * 100 + 0.5, dtype="int32")
    e = torch.empty(0, dtype=torch.float64, device=cuda)
    assert K.pix_car(e, e, 0.0, 0.0, 1e-3, 1.0, 100).numel() == 0

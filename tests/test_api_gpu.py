"""The reference-facing API (SkyMap / Tod / TodVec / make_hits / run_pcg /
NoiseSmoothedSVD) on the GPU, against reference-generated fixtures and the
CPU oracle.  GPU only."""
import math

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def mk():
    import minkasi_gb300
    return minkasi_gb300


def golden_todvec(mk, g, method):
    from minkasi_gb300.noise import NoiseSmoothedSVD
    tv = mk.TodVec()
    for k in range(int(g["ntod"])):
        tod = mk.Tod({"dat_calib": g[f"t{k}_dat"], "ipix": g[f"t{k}_ipix"]})
        tod.noise = NoiseSmoothedSVD.from_arrays(g[f"t{k}_v"], g[f"t{k}_vT"], g[f"t{k}_mywt"])
        tv.add_tod(tod)
    m = mk.SkyMap(nx=int(g["nx"]), ny=int(g["ny"]))
    tv.tod2map_method = method
    return tv, m


@pytest.mark.parametrize("method", ["atomic", "staged", "fixed", "sorted"])
def test_reference_solve_through_api(mk, gold, method):
    g = gold("solve.npz")
    tv, m = golden_todvec(mk, g, method)
    hits = mk.make_hits(tv, m)
    assert np.array_equal(hits.to_numpy(), g["hits"])
    whits = mk.make_hits(tv, m, do_weights=True)
    assert rel(whits.to_numpy(), g["whits"]) < 1e-12
    mapset = mk.Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    tv.make_rhs(rhs)
    assert rel(rhs.maps[0].to_numpy(), g["rhs"]) < 1e-12
    xr = mapset.copy()
    xr.maps[0].assign(g["xr"])
    ax = tv.dot(xr)
    assert rel(ax.maps[0].to_numpy(), g["Axr"]) < 1e-12
    x0 = rhs.copy()
    x0.clear()
    precon = mapset.copy()
    precon.maps[0].assign(g["precon"])
    xs = mk.run_pcg(rhs, x0, tv, precon, maxiter=8, verbose=False)
    assert rel(xs.maps[0].to_numpy(), g["pcg8"]) < 1e-9


def test_graph_replay_is_bitwise_equal_to_eager(mk, gold):
    g = gold("solve.npz")
    tv, m = golden_todvec(mk, g, "fixed")
    mapset = mk.Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    tv.make_rhs(rhs)
    x0 = rhs.copy()
    x0.clear()
    pre = mk.jacobi_precon(mk.make_hits(tv, m))
    a = mk.run_pcg(rhs, x0, tv, pre, maxiter=12, graph=True, verbose=False).maps[0].to_numpy()
    b = mk.run_pcg(rhs, x0, tv, pre, maxiter=12, graph=False, verbose=False).maps[0].to_numpy()
    assert np.array_equal(a, b)


def test_noise_model_u_in_path_matches_reference(mk, gold):
    g = gold("noise.npz")
    nm = mk.NoiseSmoothedSVD(g["dat"], fwhm=50.0, u_in=g["u_thin"])
    assert rel(nm.v.cpu().numpy(), g["u_v"]) < 1e-15
    assert rel(nm.vT.cpu().numpy(), g["u_vT"]) < 1e-12
    assert rel(nm.mywt.cpu().numpy(), g["u_mywt"]) < 1e-10
    assert rel(nm.apply_noise(g["x"]), g["u_dd"]) < 1e-10


def test_noise_model_gpu_svd_matches_reference_operator(mk, gold):
    g = gold("noise.npz")
    nm = mk.NoiseSmoothedSVD(g["dat"], fwhm=50.0)
    # same subspaces up to signs: |v| agrees row by row
    assert rel(np.abs(nm.v.cpu().numpy()), np.abs(g["v"])) < 1e-8
    assert rel(nm.mywt.cpu().numpy(), g["mywt"]) < 1e-8
    assert rel(nm.apply_noise(g["x"]), g["dd"]) < 1e-8
    pw = mk.NoiseSmoothedSVD(g["dat"], fwhm=50.0, prewhiten=True)
    assert np.array_equal(pw.noisevec.cpu().numpy(), g["pw_noisevec"])
    assert rel(pw.apply_noise(g["x"]), g["pw_dd"]) < 1e-8
    assert rel(nm.get_det_weights().cpu().numpy(), g["detw"]) < 1e-8


def test_module_functions_numpy_in_place(mk, gold):
    g = gold("proj.npz")
    d = g["dat"].copy()
    mk.map2tod(d, g["map"], g["ipix"], do_add=True)
    assert np.array_equal(d, g["map2tod_add"])
    m = g["map"].copy()
    mk.tod2map_omp(m, g["dat"], g["ipix"])
    assert rel(m, g["tod2map_omp"]) < 1e-13
    m2 = g["map"].copy()
    mk.tod2map_simple(m2, g["dat"], g["ipix"])
    assert rel(m2, g["tod2map_simple"]) < 1e-14


def test_bad_pixel_index_is_an_error(mk):
    tv = mk.TodVec()
    ip = np.zeros((2, 100), dtype=np.int32)
    ip[1, 50] = 10_000
    tod = mk.Tod({"dat_calib": np.ones((2, 100)), "ipix": ip})
    tv.add_tod(tod)
    m = mk.SkyMap(nx=10, ny=10)
    with pytest.raises(ValueError):
        mk.make_hits(tv, m)


def _oracle_tods(tv):
    out = []
    for t in tv.tods:
        v, vT, w = (a.cpu().numpy() for a in t.noise.operands(torch.float64))
        out.append(oracle.OracleTod(ipix=t.info["ipix"].cpu().numpy(), v=v, vT=vT, mywt=w,
                                    dat=t.info["dat_calib"].cpu().numpy()))
    return out


def test_jacobi_and_mixed_reach_1e6_checked_by_oracle(mk):
    from minkasi_gb300 import synth
    tv, m = synth.make_todvec(synth.CONFIGS["tiny"])
    mapset = mk.Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    tv.make_rhs(rhs)
    x0 = rhs.copy()
    x0.clear()
    pre = mk.jacobi_precon(mk.make_hits(tv, m))
    otods = _oracle_tods(tv)
    b = oracle.make_rhs(otods, (m.nx, m.ny))
    assert rel(rhs.maps[0].to_numpy(), b) < 1e-12

    def true_res(x):
        ax = oracle.todvec_dot(otods, x)
        return np.linalg.norm(b - ax) / np.linalg.norm(b)

    hist = []
    xj = mk.run_pcg(rhs, x0, tv, pre, maxiter=2000, tol=1e-6, verbose=False, history=hist)
    assert xj.niter < 2000
    assert true_res(xj.maps[0].to_numpy()) <= 1.05e-6
    xm = mk.run_pcg_mixed(rhs, x0, tv, pre, tol=1e-6, inner_iters=20)
    assert xm.rel_residual <= 1e-6
    assert true_res(xm.maps[0].to_numpy()) <= 1.05e-6
    # both solve the same system: maps agree once the unconstrained monopole
    # of the hit region is removed (A annihilates a constant map)
    hit = mk.make_hits(tv, m).to_numpy() > 0
    a, c = xj.maps[0].to_numpy()[hit], xm.maps[0].to_numpy()[hit]
    a, c = a - a.mean(), c - c.mean()
    assert np.linalg.norm(a - c) / np.linalg.norm(a) < 1e-3


def test_fp32_operator_per_shape_dct_engine(mk, monkeypatch):
    """The FP32 operator picks a DCT transform per TOD shape (four-step FFT,
    Bluestein on it, or cuFFT); whatever it picks, A x agrees with the same
    operator on cuFFT alone."""
    from minkasi_gb300 import synth
    from minkasi_gb300.engine import MapmakingOperator
    tv, m = synth.make_todvec(synth.CONFIGS["tiny"])
    op = tv.engine(m, torch.float32)
    assert set(op.dct_engines.values()) <= {0, 1, 2}
    x = torch.randn(m.npix, dtype=torch.float32, device="cuda")
    a = op.apply(x, torch.empty_like(x)).clone()
    monkeypatch.setenv("MINKASI_GB300_DCT", "1")
    ref_op = MapmakingOperator(tv, m, torch.float32, tod2map=op.method, rot_mode=op.rot_mode)
    assert set(ref_op.dct_engines.values()) == {1}
    b = ref_op.apply(x, torch.empty_like(x))
    assert float((a - b).abs().max() / b.abs().max()) < 1e-4


def test_mixed_replacement_policies_converge(mk):
    """Every residual-replacement interval, including replacing only when the
    recursive residual claims convergence, reaches the FP64 tolerance; a
    replacement that finds the recursive residual drifted restarts the
    search direction instead of diverging."""
    from minkasi_gb300 import synth
    tv, m = synth.make_todvec(synth.CONFIGS["tiny"])
    mapset = mk.Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    tv.make_rhs(rhs)
    x0 = rhs.copy()
    x0.clear()
    pre = mk.jacobi_precon(mk.make_hits(tv, m))
    for every in (10, 200, 10 ** 9):
        hist = []
        x = mk.run_pcg_mixed(rhs, x0, tv, pre, tol=1e-6, replace_every=every, history=hist)
        assert x.rel_residual <= 1e-6, every
        assert hist[-1]["true_rel_residual"] <= 1e-6
        assert x.outer == len(hist) and x.restarts == sum(h["restart"] for h in hist)


def test_tod2map_from_pinned_host_through_api(mk, gold):
    """SkyMap.tod2map on a pinned host timestream: chunked copies on a copy
    stream overlapped with the scatter (a small chunk makes the two-buffer
    ring wrap many times within one call and across calls)."""
    from minkasi_gb300.maps import HostStager
    g = gold("proj.npz")
    host = torch.from_numpy(np.ascontiguousarray(g["dat"])).pin_memory()
    tod = mk.Tod({"dat_calib": g["dat"], "ipix": g["ipix"]})
    m = mk.SkyMap(nx=1, ny=g["map"].size)
    m.map.copy_(torch.from_numpy(g["map"].reshape(1, -1)))
    m.tod2map(tod, host)
    assert rel(m.map.cpu().numpy().ravel(), g["tod2map_omp"].ravel()) < 1e-13
    st = HostStager(torch.device("cuda", 0))
    st.CHUNK = 1000
    flat = torch.from_numpy(g["map"].ravel().copy()).cuda()
    ip = tod.device_pix("ipix", flat.numel())
    for _ in range(3):
        st.tod2map(flat, host, ip)
    want = g["map"].ravel() + 3 * (g["tod2map_omp"].ravel() - g["map"].ravel())
    assert rel(flat.cpu().numpy(), want) < 1e-12


def test_skymap_and_polmap_write_fits(mk, tmp_path):
    """SkyMap.write: the transposed map and its CAR WCS in a FITS image;
    PolMap.write: one image per Stokes component."""
    from minkasi_gb300 import fits
    arcsec = np.pi / 180 / 3600
    lims = [3.5 - 0.002, 3.5 + 0.002, 0.3 - 0.001, 0.3 + 0.001]
    m = mk.SkyMap(lims, 2 * arcsec)
    m.map.copy_(torch.randn(m.map.shape, dtype=torch.float64))
    m.write(str(tmp_path / "sky.fits"))
    data, hdr = fits.read_image(str(tmp_path / "sky.fits"))
    assert np.array_equal(data, m.map.cpu().numpy().T)
    assert [hdr[k] for k in ("CRVAL1", "CRVAL2", "CRPIX1", "CRPIX2", "CDELT1", "CDELT2")] == list(m.wcs)
    p = mk.PolMap(lims, 2 * arcsec, "IQU")
    p.map.copy_(torch.randn(p.map.shape, dtype=torch.float64))
    p.write(str(tmp_path / "pol.fits"))
    for i, pol in enumerate("IQU"):
        d, _ = fits.read_image(str(tmp_path / f"pol_{pol}.fits"))
        assert np.array_equal(d, p.map[:, :, i].cpu().numpy().T)

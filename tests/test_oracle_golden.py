"""Pin the CPU oracle against fixtures produced by the reference code itself
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

import oracle


def test_projections_match_reference(gold):
    g = gold("proj.npz")
    ipix, dat, m = g["ipix"], g["dat"], g["map"]
    d = dat.copy()
    oracle.map2tod(d, m, ipix, do_add=True)
    assert np.array_equal(d, g["map2tod_add"])          # gather: bit-exact
    d = dat.copy()
    oracle.map2tod(d, m, ipix, do_add=False)
    assert np.array_equal(d, g["map2tod_set"])
    mm = m.copy()
    oracle.tod2map_serial(mm, dat, ipix)
    assert np.array_equal(mm, g["tod2map_simple"])      # same summation order
    mm = m.copy()
    oracle.tod2map(mm, dat, ipix)
    np.testing.assert_allclose(mm, g["tod2map_omp"], rtol=1e-12, atol=1e-12)


def test_dct1_matches_reference(gold):
    g = gold("dct.npz")
    i = 0
    while f"x{i}" in g:
        np.testing.assert_array_equal(oracle.dct1(g[f"x{i}"]), g[f"y{i}"])
        i += 1
    np.testing.assert_array_equal(oracle.dct1(g["vec_x"]), g["vec_y"])
    np.testing.assert_allclose(oracle.smooth_many_vecs(g["smooth_x"], 50.0), g["smooth_y"],
                               rtol=1e-13, atol=0)


def test_dct1_is_its_own_inverse_up_to_2n_minus_2():
    x = np.random.default_rng(1).standard_normal((3, 129))
    np.testing.assert_allclose(oracle.dct1(oracle.dct1(x)), 2 * 128 * x, rtol=1e-12, atol=1e-11)


def test_noise_model_and_apply_match_reference(gold):
    g = gold("noise.npz")
    # apply_noise with the reference's own model arrays
    np.testing.assert_allclose(oracle.apply_noise(g["v"], g["vT"], g["mywt"], g["x"]), g["dd"],
                               rtol=0, atol=1e-12 * np.abs(g["dd"]).max())
    np.testing.assert_allclose(oracle.apply_noise(g["v"], g["vT"], g["mywt"], g["x_short"]),
                               g["dd_short"], rtol=0, atol=1e-12 * np.abs(g["dd_short"]).max())
    np.testing.assert_allclose(
        oracle.apply_noise(g["pw_v"], g["pw_vT"], g["pw_mywt"], g["x"], g["pw_noisevec"]),
        g["pw_dd"], rtol=0, atol=1e-12 * np.abs(g["pw_dd"]).max())
    np.testing.assert_allclose(oracle.det_weights(g["v"], g["vT"], g["mywt"]), g["detw"], rtol=1e-12)
    # model construction through the u_in path reproduces v, vT, mywt
    v, vT, mywt, _ = oracle.noise_model(g["dat"], 50.0, u=g["u_thin"])
    np.testing.assert_allclose(v, g["u_v"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(vT, g["u_vT"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(mywt, g["u_mywt"], rtol=1e-10)
    # prewhitened model: noisevec is a median, reproduced exactly
    _, _, _, nv = oracle.noise_model(g["dat"], 50.0, prewhiten=True)
    np.testing.assert_array_equal(nv, g["pw_noisevec"])


def _tods(g):
    return [oracle.OracleTod(ipix=g[f"t{k}_ipix"], v=g[f"t{k}_v"], vT=g[f"t{k}_vT"],
                             mywt=g[f"t{k}_mywt"], dat=g[f"t{k}_dat"]) for k in range(int(g["ntod"]))]


def test_operator_rhs_hits_pcg_match_reference(gold):
    g = gold("solve.npz")
    tods = _tods(g)
    shape = (int(g["nx"]), int(g["ny"]))
    np.testing.assert_array_equal(oracle.make_hits(tods, shape), g["hits"])
    np.testing.assert_allclose(oracle.make_hits(tods, shape, do_weights=True), g["whits"], rtol=1e-12)
    b = oracle.make_rhs(tods, shape)
    np.testing.assert_allclose(b, g["rhs"], rtol=0, atol=1e-12 * np.abs(g["rhs"]).max())
    ax = oracle.todvec_dot(tods, g["xr"])
    np.testing.assert_allclose(ax, g["Axr"], rtol=0, atol=1e-12 * np.abs(g["Axr"]).max())
    x = oracle.run_pcg(g["rhs"], np.zeros(shape), lambda m: oracle.todvec_dot(tods, m),
                       g["precon"], maxiter=8)
    np.testing.assert_allclose(x, g["pcg8"], rtol=0, atol=1e-9 * np.abs(g["pcg8"]).max())


def test_truncation_lengths_match_reference(gold):
    g = gold("lens.npz")
    for n, t in zip(g["ndata"], g["truncated"]):
        assert oracle.truncate_len(int(n)) == int(t), n
    np.testing.assert_array_equal(oracle.find_good_fft_lens(1000, [2, 3, 5, 7, 11]), g["good1000"])


def test_pointing_matches_reference(gold):
    g = gold("pointing.npz")
    for k in range(int(g["ncase"])):
        ra, dec, lims = g[f"c{k}_ra"], g[f"c{k}_dec"], g[f"c{k}_lims"]
        ps, ny, cosdec = float(g[f"c{k}_pixsize"]), int(g[f"c{k}_ny"]), float(g[f"c{k}_cosdec"])
        assert np.array_equal(oracle.pix_car(ra, dec, lims, ps, ny), g[f"c{k}_car"])
        assert np.array_equal(oracle.pix_car_trunc(ra, dec, lims, ps, cosdec, ny), g[f"c{k}_trunc"])
        # points left of / below the limits: truncation toward zero differs from floor
        assert (g[f"c{k}_trunc"] != g[f"c{k}_car"]).any()


def test_wcs_car_reference_point_and_equatorial_case():
    """Unpinned (astropy absent): the CAR WCS restatement maps crval to
    crpix, and with crval on the equator it is the plain plate carree."""
    ps = 2.0 / 3600 * np.pi / 180
    for lims in ([3.5, 3.52, 0.30, 0.32], [0.7, 0.72, -0.42, -0.40]):
        w = oracle.car_wcs(lims, ps)
        p1, p2 = oracle.wcs_car_world2pix(np.array([w[0]]), np.array([w[1]]), w)
        assert abs(p1[0] - 1) < 1e-9 and abs(p2[0] - 1) < 1e-9
    w = np.array([0.0, 0.0, 1.0, 1.0, -0.01, 0.01])
    ra, dec = np.array([-0.35, 0.2]), np.array([0.25, -0.3])
    p1, p2 = oracle.wcs_car_world2pix(ra, dec, w)
    assert np.allclose(p1, 1 + ra / -0.01, rtol=0, atol=1e-9)
    assert np.allclose(p2, 1 + dec / 0.01, rtol=0, atol=1e-9)


def test_pol_projections_invert_mul_match_reference(gold):
    g = gold("pol.npz")
    ipix, tg, dat = g["ipix"], g["twogamma"], g["dat"]
    for tag in ("IQU", "QU"):
        for add in (0, 1):
            d = dat.copy()
            oracle.polmap2tod(d, g[f"map_{tag}"], tag, tg, ipix, bool(add))
            assert np.abs(d - g[f"m2t_{tag}_{add}"]).max() < 1e-12 * np.abs(g[f"m2t_{tag}_{add}"]).max()
    for tag in ("IQU", "QU", "QU_PRECON", "IQU_PRECON"):
        m = g[f"t2m_in_{tag}"].copy()
        oracle.tod2polmap(m, dat, tag, tg, ipix)
        assert np.abs(m - g[f"t2m_{tag}"]).max() < 1e-12 * np.abs(g[f"t2m_{tag}"]).max()
    for tag in ("IQU", "QU"):
        h = np.zeros_like(g[f"hits_{tag}"])
        for k in range(2):
            oracle.tod2polmap(h, np.ones(dat.shape), tag + "_PRECON", g[f"hits_t{k}_twogamma"],
                              g[f"hits_t{k}_ipix"])
        assert np.abs(h - g[f"hits_{tag}"]).max() < 1e-12 * np.abs(h).max()
        inv = oracle.pol_invert(g[f"hits_{tag}"], tag + "_PRECON")
        assert np.allclose(inv, g[f"inv_{tag}"], rtol=1e-9, atol=1e-12 * np.abs(inv).max())
        mul = oracle.pol_precon_mul(g[f"inv_{tag}"], g[f"mulx_{tag}"], tag + "_PRECON")
        assert np.allclose(mul, g[f"mul_{tag}"], rtol=1e-12, atol=0)
        assert (h != 0).any()


def test_cuts_stripes_binned_match_reference(gold):
    g = gold("tsmodel.npz")
    dat = g["dat"]
    # cuts: imap from the mask, gather and scatter through the reference's C
    parts = []
    for d in range(dat.shape[0]):
        edges = np.where(np.diff(np.r_[True, g["cut_mask"][d], True]))[0]
        for a, b in zip(edges[::2], edges[1::2]):
            parts.append(np.arange(d * dat.shape[1] + a, d * dat.shape[1] + b))
    imap = np.concatenate(parts)
    assert np.array_equal(imap, g["cut_imap"])
    v = np.zeros(imap.size)
    oracle.cuts_gather(v, dat, imap)
    assert np.array_equal(v, g["cut_map"])
    for add in (0, 1):
        d = dat.copy()
        oracle.cuts_scatter(d, g["cut_vals"], imap, bool(add))
        assert np.array_equal(d, g[f"cut_m2t_{add}"])
    # stripes: segment edges, map2tod, and tod2map as its transpose
    lims = oracle.stripe_edges(dat.shape[1], g["ctime"], seg_len=170)
    assert np.array_equal(lims, g["stripe_inds"])
    for add in (0, 1):
        d = dat.copy()
        oracle.stripes_map2tod(d, g["stripe_pars"], lims, bool(add))
        assert np.array_equal(d, g[f"stripe_m2t_{add}"])
    p = np.zeros_like(g["stripe_pars"])
    oracle.stripes_tod2map(p, dat, lims)
    m = np.zeros_like(dat)
    oracle.stripes_map2tod(m, g["stripe_pars"], lims, False)
    assert abs(np.sum(m * dat) - np.sum(p * g["stripe_pars"])) < 1e-10 * abs(np.sum(m * dat))
    # binned: map2tod, and the histogram where the reference's buffered add agrees
    for add in (0, 1):
        d = dat.copy()
        oracle.binned_map2tod(d, g["bin_pars"], g["az"], (0, 2 * np.pi), int(g["nbin"]), bool(add))
        assert np.array_equal(d, g[f"bin_m2t_{add}"])
    nb = int(g["nbin_unique"])
    p1 = np.zeros((dat.shape[0], nb))
    oracle.binned_tod2map(p1, dat, g["az_unique"], (0, 2 * np.pi), nb)
    inds = np.asarray(g["az_unique"] * (nb / (2 * np.pi)), dtype="int64")
    once = np.bincount(inds, minlength=nb) == 1
    assert np.array_equal(p1[:, once], g["bin_t2m_unique"][:, once])
    assert (~once[inds]).any()  # some bins repeat: there the reference keeps one sample

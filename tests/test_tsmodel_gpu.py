"""Cuts and timestream-model members of a Mapset (mk_cuts_*, mk_stripes_*,
mk_binned_*, CutsCompact, tsStripes, tsBinnedAz, tsModel) against the
reference's own outputs (tsmodel.npz) and the oracle.  GPU only."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda", 0)
TWO_PI = 2 * np.pi


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    return t.to(dtype) if dtype is not None else t


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def K():
    from minkasi_gb300 import kernels
    return kernels


def test_cuts_kernels_bit_exact(K, gold):
    g = gold("tsmodel.npz")
    imap = dev(g["cut_imap"])
    v = torch.zeros(imap.numel(), dtype=torch.float64, device=cuda)
    K.cuts_gather(v, dev(g["dat"]), imap, do_add=True)
    assert np.array_equal(v.cpu().numpy(), g["cut_map"])
    for add in (0, 1):
        d = dev(g["dat"])
        K.cuts_scatter(d, dev(g["cut_vals"]), imap, do_add=bool(add))
        assert np.array_equal(d.cpu().numpy(), g[f"cut_m2t_{add}"])


def test_stripes_kernels(K, gold):
    g = gold("tsmodel.npz")
    lims = dev(g["stripe_inds"].astype(np.int64))
    for add in (0, 1):
        d = dev(g["dat"])
        K.stripes_map2tod(d, dev(g["stripe_pars"]), lims, do_add=bool(add))
        assert np.array_equal(d.cpu().numpy(), g[f"stripe_m2t_{add}"])
    for add in (0, 1):
        p0 = np.random.default_rng(add).standard_normal(g["stripe_pars"].shape)
        ref = p0.copy()
        oracle.stripes_tod2map(ref, g["dat"], g["stripe_inds"], bool(add))
        p = dev(p0)
        K.stripes_tod2map(p, dev(g["dat"]), lims, do_add=bool(add))
        assert rel(p.cpu().numpy(), ref) < 1e-13
    p = torch.zeros(g["stripe_pars"].shape, dtype=torch.float32, device=cuda)
    K.stripes_tod2map(p, dev(g["dat"], torch.float32), lims, do_add=False)
    ref = np.zeros_like(g["stripe_pars"])
    oracle.stripes_tod2map(ref, g["dat"], g["stripe_inds"], False)
    assert rel(p.cpu().numpy(), ref) < 1e-5


def test_binned_kernels(K, gold):
    g = gold("tsmodel.npz")
    az, nbin = dev(g["az"]), int(g["nbin"])
    for add in (0, 1):
        d = dev(g["dat"])
        K.binned_map2tod(d, dev(g["bin_pars"]), az, (0, TWO_PI), do_add=bool(add))
        assert np.array_equal(d.cpu().numpy(), g[f"bin_m2t_{add}"])
    ref = np.zeros((g["dat"].shape[0], nbin))
    oracle.binned_tod2map(ref, g["dat"], g["az"], (0, TWO_PI), nbin)
    p = torch.zeros((g["dat"].shape[0], nbin), dtype=torch.float64, device=cuda)
    K.binned_tod2map(p, dev(g["dat"]), az, (0, TWO_PI), do_add=False)
    assert rel(p.cpu().numpy(), ref) < 1e-12
    # more bins than the shared-memory histogram holds (global atomics); the
    # reference where its buffered add agrees (bins hit by one sample)
    nb = int(g["nbin_unique"])
    p1 = torch.zeros((g["dat"].shape[0], nb), dtype=torch.float64, device=cuda)
    K.binned_tod2map(p1, dev(g["dat"]), dev(g["az_unique"]), (0, TWO_PI), do_add=True)
    inds = np.asarray(g["az_unique"] * (nb / TWO_PI), dtype="int64")
    once = np.bincount(inds, minlength=nb) == 1
    assert np.array_equal(p1.cpu().numpy()[:, once], g["bin_t2m_unique"][:, once])
    ref1 = np.zeros((g["dat"].shape[0], nb))
    oracle.binned_tod2map(ref1, g["dat"], g["az_unique"], (0, TWO_PI), nb)
    assert rel(p1.cpu().numpy(), ref1) < 1e-12


def test_cutscompact_and_prior_from_skymap(gold):
    import minkasi_gb300 as mk
    g = gold("tsmodel.npz")
    tod = mk.Tod({"dat_calib": g["dat"], "fname": "t0"})
    cc = mk.CutsCompact(tod)
    cc.cuts_from_array(g["cut_mask"])
    cc.get_imap()
    assert np.array_equal(cc.imap.cpu().numpy(), g["cut_imap"])
    cc.tod2map(tod, dev(g["dat"]))
    assert np.array_equal(cc.map.cpu().numpy(), g["cut_map"])
    cc.map.copy_(dev(g["cut_vals"]))
    d = dev(g["dat"])
    cc.map2tod(tod, d, do_add=True)
    assert np.array_equal(d.cpu().numpy(), g["cut_m2t_1"])
    c2 = cc.copy()
    c2.axpy(cc, 2.0)
    ss = float(np.sum(g["cut_vals"] ** 2))
    assert abs(c2.dot(cc) - 3 * ss) < 1e-9 * ss
    # a prior from a map that is non-zero on 5 of its pixels
    rng = np.random.default_rng(3)
    ipix = rng.integers(0, 40, size=g["dat"].shape).astype(np.int32)
    t2 = mk.Tod({"dat_calib": g["dat"], "fname": "t1", "ipix": ipix})
    m = mk.SkyMap(nx=1, ny=40)
    m.map[0, :5] = torch.arange(1, 6, dtype=torch.float64)
    prior = t2.prior_from_skymap(m)
    assert prior.imap.numel() == int((ipix < 5).sum())
    want = 1.0 / (ipix.ravel()[prior.imap.cpu().numpy()] + 1.0) ** 2
    assert np.allclose(prior.map.cpu().numpy(), want, rtol=1e-15)


def test_tsstripes_and_binned_classes(gold):
    import minkasi_gb300 as mk
    g = gold("tsmodel.npz")
    tod = mk.Tod({"dat_calib": g["dat"], "fname": "t0", "ctime": g["ctime"], "az": g["az"]})
    st = mk.tsStripes(tod, seg_len=170)
    assert np.array_equal(st.inds, g["stripe_inds"])
    st.params.copy_(dev(g["stripe_pars"]))
    d = dev(g["dat"])
    st.map2tod(tod, d, do_add=True)
    assert np.array_equal(d.cpu().numpy(), g["stripe_m2t_1"])
    st.set_prior_from_corr(g["stripe_corr"], thresh=0.5)
    assert rel(st.params.cpu().numpy(), g["stripe_prior"]) < 1e-12
    x, ax = mk.tsStripes(tod, seg_len=170), mk.tsStripes(tod, seg_len=170)
    x.params.copy_(dev(g["stripe_x"]))
    ax.params.copy_(dev(g["stripe_ax0"]))
    st.apply_prior(x, ax)
    assert rel(ax.params.cpu().numpy(), g["stripe_ax"]) < 1e-11
    bz = mk.tsBinnedAz(tod, nbin=int(g["nbin"]))
    bz.params.copy_(dev(g["bin_pars"]))
    d = dev(g["dat"])
    bz.map2tod(tod, d, do_add=False)
    assert np.array_equal(d.cpu().numpy(), g["bin_m2t_0"])


def test_mixed_mapset_operator_matches_oracle(gold):
    """A x for a Mapset of a sky map and a destriper tsModel, through
    TodVec.dot (per-TOD path), against the oracle's operator."""
    import minkasi_gb300 as mk
    from minkasi_gb300.noise import NoiseSmoothedSVD
    g = gold("solve.npz")
    nx, ny = int(g["nx"]), int(g["ny"])
    ntod = int(g["ntod"])
    tv = mk.TodVec()
    for k in range(ntod):
        nd = g[f"t{k}_dat"].shape[1]
        tod = mk.Tod({"dat_calib": g[f"t{k}_dat"], "ipix": g[f"t{k}_ipix"], "fname": f"t{k}",
                      "ctime": np.arange(nd) * 0.01})
        tod.noise = NoiseSmoothedSVD.from_arrays(g[f"t{k}_v"], g[f"t{k}_vT"], g[f"t{k}_mywt"])
        tv.add_tod(tod)
    x = mk.Mapset()
    x.add_map(mk.SkyMap(nx=nx, ny=ny))
    x.add_map(mk.tsModel(tv, mk.tsStripes, seg_len=60))
    rng = np.random.default_rng(5)
    x.maps[0].map.copy_(dev(rng.standard_normal((nx, ny))))
    for k in range(ntod):
        p = x.maps[1].data[f"t{k}"].params
        p.copy_(dev(rng.standard_normal(tuple(p.shape))))
    y = tv.dot(x)
    xm = x.maps[0].map.cpu().numpy().ravel()
    want_map = np.zeros(nx * ny)
    for k in range(ntod):
        ip = g[f"t{k}_ipix"]
        lims = x.maps[1].data[f"t{k}"].inds
        pars = x.maps[1].data[f"t{k}"].params.cpu().numpy()
        tmp = np.zeros(ip.shape)
        oracle.map2tod(tmp, xm, ip, False)
        oracle.stripes_map2tod(tmp, pars, lims, True)
        tmp = oracle.apply_noise(g[f"t{k}_v"], g[f"t{k}_vT"], g[f"t{k}_mywt"], tmp)
        oracle.tod2map(want_map, tmp, ip)
        ps = np.zeros_like(pars)
        oracle.stripes_tod2map(ps, tmp, lims)
        assert rel(y.maps[1].data[f"t{k}"].params.cpu().numpy(), ps) < 1e-10
    assert rel(y.maps[0].map.cpu().numpy().ravel(), want_map) < 1e-10
    # the operator is symmetric: <x, A z> = <z, A x>
    z = x.copy()
    z.maps[0].map.copy_(dev(rng.standard_normal((nx, ny))))
    az = tv.dot(z)
    a, b = x.dot(az), z.dot(y)
    assert abs(a - b) < 1e-10 * abs(a)

"""Polarized projections (mk_polmap2tod, mk_tod2polmap, mk_pol_precon_mul)
and the PolMap API against the reference's own outputs (pol.npz).  GPU only."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda", 0)


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


@pytest.mark.parametrize("form", ["twogamma", "sincos"])
def test_polmap2tod_matches_reference(K, gold, form):
    g = gold("pol.npz")
    tg = dev(g["twogamma"])
    angle = tg if form == "twogamma" else K.pol_sincos(tg)
    for tag in ("IQU", "QU"):
        for add in (0, 1):
            d = dev(g["dat"])
            K.polmap2tod(d, dev(g[f"map_{tag}"]), tag, angle, dev(g["ipix"]), bool(add))
            assert rel(d.cpu().numpy(), g[f"m2t_{tag}_{add}"]) < 1e-12, (tag, add)


@pytest.mark.parametrize("form", ["twogamma", "sincos"])
def test_tod2polmap_all_modes_match_reference(K, gold, form):
    g = gold("pol.npz")
    tg = dev(g["twogamma"])
    angle = tg if form == "twogamma" else K.pol_sincos(tg)
    for tag in ("IQU", "QU", "QU_PRECON", "IQU_PRECON"):
        m = dev(g[f"t2m_in_{tag}"])
        K.tod2polmap(m, dev(g["dat"]), tag, angle, dev(g["ipix"]))
        assert rel(m.cpu().numpy(), g[f"t2m_{tag}"]) < 1e-12, tag


def test_pol_fp32(K, gold):
    g = gold("pol.npz")
    angle = K.pol_sincos(dev(g["twogamma"]), torch.float32)
    d = dev(g["dat"], torch.float32)
    K.polmap2tod(d, dev(g["map_IQU"], torch.float32), "IQU", angle, dev(g["ipix"]), True)
    assert rel(d.cpu().numpy(), g["m2t_IQU_1"]) < 2e-6
    m = dev(g["t2m_in_IQU_PRECON"], torch.float32)
    K.tod2polmap(m, dev(g["dat"], torch.float32), "IQU_PRECON", angle, dev(g["ipix"]))
    assert rel(m.cpu().numpy(), g["t2m_IQU_PRECON"]) < 2e-5


def test_pol_bad_arguments(K, gold):
    g = gold("pol.npz")
    with pytest.raises(K._lib.MkError):  # no map2tod for PRECON modes, as in the reference
        K.polmap2tod(dev(g["dat"]), dev(g["t2m_in_QU_PRECON"]), "QU_PRECON", dev(g["twogamma"]),
                     dev(g["ipix"]))
    with pytest.raises(K._lib.MkError):  # the twogamma form is FP64 only
        K.polmap2tod(dev(g["dat"], torch.float32), dev(g["map_QU"], torch.float32), "QU",
                     dev(g["twogamma"]), dev(g["ipix"]))


@pytest.mark.parametrize("tag", ["IQU", "QU"])
def test_polmap_hits_invert_mul_and_projections(gold, tag):
    import minkasi_gb300 as mk
    g = gold("pol.npz")
    nx, ny = int(g["nx"]), int(g["ny"])
    tv = mk.TodVec()
    for k in range(2):
        tv.add_tod(mk.Tod({"dat_calib": g["dat"] * (k + 1), "ipix": g[f"hits_t{k}_ipix"],
                           "twogamma_saved": g[f"hits_t{k}_twogamma"]}))
    m = mk.PolMap(None, 0.0, tag, nx=nx, ny=ny)
    hits = mk.make_hits(tv, m)
    assert hits.poltag == tag + "_PRECON"
    assert rel(hits.map.cpu().numpy(), g[f"hits_{tag}"]) < 1e-12
    inv = hits.copy()
    inv.invert()
    ref = g[f"inv_{tag}"]
    assert np.allclose(inv.map.cpu().numpy(), ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())
    x = mk.PolMap(None, 0.0, tag, nx=nx, ny=ny)
    x.assign(g[f"mulx_{tag}"])
    inv.assign(g[f"inv_{tag}"])
    assert rel((inv * x).map.cpu().numpy(), g[f"mul_{tag}"]) < 1e-13
    # map2tod / tod2map through the map object (tod.info carries ipix and twogamma)
    m.assign(g[f"map_{tag}"])
    tod = mk.Tod({"dat_calib": g["dat"], "ipix": g["ipix"], "twogamma_saved": g["twogamma"]})
    d = dev(g["dat"])
    m.map2tod(tod, d, do_add=True)
    assert rel(d.cpu().numpy(), g[f"m2t_{tag}_1"]) < 1e-12
    acc = mk.PolMap(None, 0.0, tag, nx=nx, ny=ny)
    acc.assign(g[f"t2m_in_{tag}"])
    acc.tod2map(tod, g["dat"])
    assert rel(acc.map.cpu().numpy(), g[f"t2m_{tag}"]) < 1e-12
    assert abs(acc.dot(acc) - float(np.sum(g[f"t2m_{tag}"] ** 2))) < 1e-10 * float(np.sum(g[f"t2m_{tag}"] ** 2))

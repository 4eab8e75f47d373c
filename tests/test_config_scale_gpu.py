"""The operator on the benchmark configurations' own shapes, against the
oracle (the FP64 CPU restatement of minkasi/tods/core.py:967-1047 and
minkasi/mapmaking/tod2map.py:343-400):

* the single-TOD configuration in full: 64 detectors x 65,341 samples onto
  a 256 x 256 map at 2";
* two TODs of the 32-TOD configuration (256 detectors, 1024 x 1024 map at
  1"): 130,978 samples, whose DCT length 2(n-1) factors into small primes,
  and 144,278 samples, where 2(n-1) = 2 * 7 * 20611 and the FP32 DCT runs
  Bluestein's algorithm.

TodVec.dot, make_rhs and make_hits run through the public API in FP64 and
are held to 1e-12 relative (max error over max value; hits exactly).  The
FP32 operator (FP32 projections and DCT-I, 3xTF32 tensor-core or FP32 cuBLAS
rotation) is held to 1e-5 relative L2 against the FP64 oracle, with each
FP32 DCT engine (four-step FFT with Bluestein, cuFFT).  GPU only."""
import os

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
cuda = torch.device("cuda", 0)
WORKERS = os.cpu_count() or 1


def rel_max(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _case(name):
    import minkasi_gb300 as mk
    from minkasi_gb300 import synth
    from minkasi_gb300.tods import Tod, TodVec
    if name == "c1":
        cfg = synth.CONFIGS["c1"]
        picks = [(0,) + synth.tod_shapes(cfg)[0]]
    else:
        cfg = synth.CONFIGS["c2"]
        picks = [(0, 256, 130978), (1, 256, 144278)]
    tv = TodVec()
    for k, ndet, n in picks:
        info = synth.make_tod_info(cfg, k, ndet, n, cuda, with_radec=False)
        tod = Tod(info)
        tod.set_noise()
        tv.add_tod(tod)
    m = mk.SkyMap(nx=cfg.nx, ny=cfg.ny, device=cuda)
    otods = []
    for t in tv.tods:
        v, vT, w = (a.cpu().numpy() for a in t.noise.operands(torch.float64))
        otods.append(oracle.OracleTod(ipix=t.info["ipix"].cpu().numpy(), v=v, vT=vT, mywt=w,
                                      dat=t.info["dat_calib"].cpu().numpy()))
    return tv, m, otods


@pytest.fixture(scope="module", params=["c1", "c2_two_tods"])
def case(request):
    return _case(request.param)


def test_fp64_dot_rhs_hits_at_config_scale(case):
    import minkasi_gb300 as mk
    tv, m, otods = case
    shape = (m.nx, m.ny)
    hits = mk.make_hits(tv, m).to_numpy()
    assert np.array_equal(hits, oracle.make_hits(otods, shape))
    hit = hits.reshape(-1) > 0
    mapset = mk.Mapset()
    mapset.add_map(m)
    rhs = mapset.copy()
    tv.make_rhs(rhs)
    b_ref = oracle.make_rhs(otods, shape, workers=WORKERS)
    assert rel_max(rhs.maps[0].to_numpy(), b_ref) < 1e-12
    x = np.where(hit, np.random.default_rng(3).standard_normal(m.npix), 0.0).reshape(shape)
    xs = mapset.copy()
    xs.maps[0].assign(x)
    ax = tv.dot(xs).maps[0].to_numpy()
    ax_ref = oracle.todvec_dot(otods, x, workers=WORKERS)
    assert rel_max(ax, ax_ref) < 1e-12


@pytest.mark.parametrize("dct_engine", ["0", "1"])
@pytest.mark.parametrize("rot_mode", [1, 2])
def test_fp32_operator_at_config_scale(case, dct_engine, rot_mode, monkeypatch):
    from minkasi_gb300.engine import MapmakingOperator
    tv, m, otods = case
    monkeypatch.setenv("MINKASI_GB300_DCT", dct_engine)
    op = MapmakingOperator(tv, m, torch.float32, tod2map="atomic", rot_mode=rot_mode)
    # the plans report 0 (four-step FFT), 2 (four-step through Bluestein) or 1 (cuFFT)
    assert set(op.dct_engines.values()) <= ({1} if dct_engine == "1" else {0, 2})
    hit = op.hits().cpu().numpy() > 0
    x = np.where(hit, np.random.default_rng(4).standard_normal(m.npix), 0.0).astype(np.float32)
    out = op.apply(torch.from_numpy(x).to(cuda), torch.empty(m.npix, dtype=torch.float32, device=cuda))
    ax_ref = oracle.todvec_dot(otods, x.astype(np.float64).reshape(m.nx, m.ny), workers=WORKERS)
    err = rel_l2(out.cpu().double().numpy(), ax_ref.reshape(-1))
    assert err < 1e-5, err
    op.release()

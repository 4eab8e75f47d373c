"""The tcgen05 3xTF32 tensor-core rotation against an FP64 reference product
and against the cuBLAS FP32 rotation, alone and inside apply_noise.  GPU only.

Tolerance: 3xTF32 keeps FP32-level accuracy; max |R - R64| / max |R64| <= 5e-6.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
cuda = torch.device("cuda", 0)


@pytest.fixture(scope="module")
def K():
    from minkasi_gb300 import kernels
    return kernels


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("ndet", [32, 64, 128, 256])
@pytest.mark.parametrize("ncol", [128, 1000, 4097])
def test_tc_rotation_matches_fp64(K, ndet, ncol):
    rng = np.random.default_rng(ndet * 7 + ncol)
    A = rng.standard_normal((ndet, ndet)).astype(np.float32)
    X = rng.standard_normal((ndet, ncol)).astype(np.float32)
    ref = A.astype(np.float64) @ X.astype(np.float64)
    plan = K.NoisePlan(ndet, ncol, torch.float32)
    At, Xt = torch.from_numpy(A).to(cuda), torch.from_numpy(X).to(cuda)
    R2 = plan.rotate(At, Xt, rot_mode=2).cpu().numpy()
    assert plan.status() == 0
    R1 = plan.rotate(At, Xt, rot_mode=1).cpu().numpy()
    assert rel(R1, ref) < 5e-6
    assert rel(R2, ref) < 5e-6


def test_tc_apply_noise_matches_golden(K, gold):
    g = gold("noise.npz")
    x = g["x"]
    # pad the 10-detector fixture into a 32-detector block (identity elsewhere)
    nd = 32
    v = np.eye(nd)
    vT = np.eye(nd)
    w = np.zeros((nd, x.shape[1]))
    xx = np.zeros((nd, x.shape[1]))
    v[:10, :10], vT[:10, :10], w[:10], xx[:10] = g["v"], g["vT"], g["mywt"], x
    plan = K.NoisePlan(nd, x.shape[1], torch.float32)
    f = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(cuda)
    dd = plan.apply(f(v), f(vT), f(w), f(xx), rot_mode=2).cpu().numpy()
    assert plan.status() == 0
    assert rel(dd[:10], g["dd"]) < 2e-5


@pytest.mark.parametrize("dct", ["0", "1"])
def test_noise_group_equals_per_tod_filter(monkeypatch, dct):
    """The one-call filter over all TODs (rotations of all TODs with one
    detector count in one tensor-core launch, in place) gives bit for bit
    what the per-TOD apply_noise gives, on TODs of 32 and 64 detectors with
    untruncated lengths (so some run Bluestein's algorithm), with the
    four-step FFT and with cuFFT plans."""
    from dataclasses import replace
    from minkasi_gb300 import synth
    from minkasi_gb300.engine import MapmakingOperator
    monkeypatch.setenv("MINKASI_GB300_DCT", dct)
    cfg = replace(synth.CONFIGS["tiny"], ntod=5, ndet_choices=(32, 64), nsamp_range=(3000, 9000),
                  truncate=False)
    tv, m = synth.make_todvec(cfg)
    op = MapmakingOperator(tv, m, torch.float32, tod2map="atomic", rot_mode=2)
    if dct == "0":
        assert set(op.dct_engines.values()) <= {0, 2} and 2 in op.dct_engines.values()
    else:
        assert set(op.dct_engines.values()) == {1}
    grp = op._noise_group()
    assert grp is not None
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(op.tmp.shape, generator=g, dtype=torch.float32, device="cuda")
    op.tmp.copy_(x)
    op.noise_all()
    grouped = op.tmp.clone()
    assert grp.status() == 0
    op.tmp.copy_(x)
    for (v, vT, w), view, dims in zip(op.ops, op.views(op.tmp), op.dims):
        op.plans[dims].apply(v, vT, w, view, out=view, rot_mode=2)
    assert torch.equal(grouped, op.tmp)

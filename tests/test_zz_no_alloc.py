"""mk_tod2map_fixed_noalloc: the tod2map for callers that cannot allocate
device memory (its accumulator is a device array built into the library).

Called through the C ABI and checked against mk_tod2map_fixed with caller
scratch, on two calls in a row: the second call must see the built-in
scratch left clean by the first.  Its data are a million times smaller than
the first call's, so a header left over from the first call (its max|dat|,
hence its fixed-point shift) would cost the second call about 20 bits and
show far above the tolerance.  Both paths run the same arithmetic, so they
must agree bit for bit; both are also held to the other tod2map parity
tests' 1e-13 relative against the oracle's serial sum.
Collected last on purpose.  GPU only.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
cuda = torch.device("cuda", 0)


def _case(seed, ndet, ndata, npix):
    rng = np.random.default_rng(seed)
    walk = np.cumsum(rng.integers(-1, 2, size=(ndet, ndata)), axis=1) // 3
    ipix = np.mod(walk + rng.integers(0, npix, size=(ndet, 1)), npix).astype(np.int32)
    dat = rng.standard_normal((ndet, ndata))
    return ipix, dat


def test_noalloc_matches_scratch_variant_twice():
    import oracle
    from minkasi_gb300 import _lib, kernels as K

    h = _lib.load()
    vp = ctypes.c_void_p
    stream = vp(torch.cuda.current_stream().cuda_stream)
    npix = 1 << 16
    outs = []
    for call, (seed, scale) in enumerate(((11, 1.0), (12, 1e-6))):
        ipix, dat = _case(seed, 12, 30_001, npix)
        dat *= scale
        gi = torch.from_numpy(ipix).to(cuda)
        gd = torch.from_numpy(dat).to(cuda)
        hmax = int(np.bincount(ipix.ravel(), minlength=npix).max())
        base = torch.from_numpy(np.random.default_rng(seed + 100).standard_normal(npix) * scale).to(cuda)
        ref = base.clone()
        scratch = K.FixedScratch(npix)
        assert h.mk_tod2map_fixed(vp(ref.data_ptr()), vp(gd.data_ptr()), vp(gi.data_ptr()), 12, 30_001,
                                  npix, hmax, _lib.MK_F64, vp(scratch.buf.data_ptr()), stream) == 0
        got = base.clone()
        rc = h.mk_tod2map_fixed_noalloc(vp(got.data_ptr()), vp(gd.data_ptr()), vp(gi.data_ptr()), 12,
                                        30_001, npix, hmax, _lib.MK_F64, stream)
        assert rc == 0, h.mk_last_error()
        torch.cuda.synchronize()
        r, g = ref.cpu().numpy(), got.cpu().numpy()
        assert np.array_equal(g, r), call
        want = base.cpu().numpy()
        oracle.tod2map_serial(want, dat, ipix)
        assert np.abs(g - want).max() <= 1e-13 * np.abs(want).max(), call
        outs.append(g)
    assert not np.array_equal(outs[0], outs[1])


def test_noalloc_rejects_maps_above_the_limit():
    from minkasi_gb300 import _lib

    h = _lib.load()
    too_big = 4194304 + 1
    rc = h.mk_tod2map_fixed_noalloc(None, None, None, 1, 1, too_big, 1, _lib.MK_F64, None)
    assert rc == _lib.MK_ERR_ARG
    assert b"limit" in h.mk_last_error()
    rc = h.mk_tod2map_fixed_noalloc(None, None, None, 1, 1, -5, 1, _lib.MK_F64, None)
    assert rc == _lib.MK_ERR_ARG
    assert b"negative npix" in h.mk_last_error()

"""Host-side checks that need no GPU: the C-ABI library loads and exports
every entry point include/mkgpu.h declares, truncation and synthetic-shape
logic, TOD partitioning."""
import ctypes
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_header_symbol():
    from minkasi_gb300 import _lib
    h = _lib.load()
    declared = _lib.header_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(h, name), name           # dlsym succeeds
        assert name in _lib.SIGNATURES, name     # and the binding covers it
    assert h.mk_version() >= 1
    assert h.mk_reduce_scratch_bytes() > 0       # pure host query, no device work


def test_library_is_built_for_sm103a():
    # the build passes one -gencode for compute_103a/sm_103a
    from minkasi_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_argument_errors_need_no_gpu():
    from minkasi_gb300 import _lib
    h = _lib.load()
    assert h.mk_map2tod(None, None, None, 1, 1, 1, 7, 0, None) == _lib.MK_ERR_ARG
    assert b"dtype" in h.mk_last_error()
    nb = ctypes.c_size_t(0)
    assert h.mk_dct1_workspace_bytes(4, 1, 0, ctypes.byref(nb)) == _lib.MK_ERR_ARG
    assert h.mk_tod2map_fixed(None, None, None, 1, 1, 1, 0, 0, None, None) == _lib.MK_ERR_ARG


def _smooth(x):
    for p in (2, 3, 5, 7, 11):
        while x % p == 0:
            x //= p
    return x == 1


def test_dct_plan_selection_needs_no_gpu():
    """Which transform an FP32 DCT plan uses, decided on the host: the
    four-step split of 2(n-1) when it factors into 2..11, otherwise
    Bluestein's smallest splittable smooth M >= 3(n-1) (only outputs
    0..n-1 are kept and the even extension is symmetric, so the lags span
    3(n-1) values), cuFFT beyond 1536 x 1536 or when selected."""
    from minkasi_gb300 import kernels as K
    assert K.dct_engine() == 0
    d = K.dct_describe(130978)                 # 2 * 3^5 * 7^2 * 11
    assert d == {"engine": 0, "L": 261954, "L1": d["L1"], "L2": d["L2"]}
    assert d["L1"] * d["L2"] == 261954 and max(d["L1"], d["L2"]) <= 1536 and d["L1"] > 1
    assert K.dct_describe(2) == {"engine": 0, "L": 2, "L1": 2, "L2": 1}
    for n in (38, 1000, 465551, 144278):         # 2(n-1) has 37, 37, 9311, 72139
        d = K.dct_describe(n)
        assert d["engine"] == 2 and _smooth(d["L"]) and d["L"] >= 3 * (n - 1)
        # and the smallest such length with a split into two parts <= 1536
        assert not any(_smooth(M) and any(M % a == 0 and M // a <= 1536 for a in range(2, 1537))
                       for M in range(3 * (n - 1), d["L"]))
        assert d["L1"] * d["L2"] == d["L"] and max(d["L1"], d["L2"]) <= 1536
    assert K.dct_describe(10 ** 7)["engine"] == 1
    try:
        K.set_dct_engine(2)
        assert K.dct_describe(465551)["engine"] == 1 and K.dct_describe(130978)["engine"] == 0
        K.set_dct_engine(1)
        assert K.dct_describe(130978) == {"engine": 1, "L": 261954, "L1": 0, "L2": 0}
    finally:
        K.set_dct_engine(0)


def test_dct_engine_choice_host_logic(monkeypatch):
    """The per-shape transform choice without a GPU: FP64 operators keep the
    current engine, MINKASI_GB300_DCT forces one, and with_dct_engine
    restores the engine even when its body raises."""
    import torch
    from types import SimpleNamespace
    from minkasi_gb300 import kernels as K
    from minkasi_gb300.autotune import choose_dct_engines, with_dct_engine
    shapes = [(16, 3529), (32, 4097)]
    assert choose_dct_engines(SimpleNamespace(dtype=torch.float64), shapes) == {s: (0, 0) for s in shapes}
    monkeypatch.setenv("MINKASI_GB300_DCT", "1")
    assert choose_dct_engines(SimpleNamespace(dtype=torch.float32), shapes) == {s: (1, 0) for s in shapes}
    assert with_dct_engine(2, lambda: K.dct_describe(465551)["engine"]) == 1
    assert K.dct_engine() == 0
    # a split rank selects another L1 x L2 of the same length, and is restored
    d0 = K.dct_describe(130978)
    d1 = with_dct_engine((0, 1), lambda: K.dct_describe(130978))
    assert d0["L"] == d1["L"] and d0["L1"] * d0["L2"] == d1["L1"] * d1["L2"] == d0["L"]
    assert (d0["L1"], d0["L2"]) != (d1["L1"], d1["L2"])
    assert K.fft4_split() == 0

    def boom():
        assert K.dct_engine() == 1
        raise RuntimeError("inside")
    with pytest.raises(RuntimeError):
        with_dct_engine(1, boom)
    assert K.dct_engine() == 0


def test_truncation_matches_reference(gold):
    from minkasi_gb300 import truncate
    g = gold("lens.npz")
    for n, t in zip(g["ndata"], g["truncated"]):
        assert truncate.truncated_length(int(n)) == int(t)
    info = {"dat_calib": np.zeros((3, 1025)), "ipix": np.zeros((3, 1025), np.int32), "x": 5}
    truncate.truncate_tod(info)
    assert info["dat_calib"].shape == (3, g["truncated"][list(g["ndata"]).index(1025)])


def test_synth_shapes_are_seeded_and_smooth():
    from minkasi_gb300 import synth, truncate
    a = synth.tod_shapes(synth.CONFIGS["c2"])
    b = synth.tod_shapes(synth.CONFIGS["c2"])
    assert a == b and len(a) == 32
    for ndet, n in a:
        assert ndet == 256 and (1 << 17) - 2000 <= n <= (1 << 19)
        assert truncate.truncated_length(n) == n   # already FFT friendly
    c4 = synth.tod_shapes(synth.CONFIGS["c4"])
    assert len(c4) == 200 and set(d for d, _ in c4) <= {32, 64, 128, 256}


def test_synth_pointing_in_range_on_cpu():
    import torch
    from minkasi_gb300 import synth
    cfg = synth.CONFIGS["tiny"]
    info = synth.make_tod_info(cfg, 0, 8, 3001, torch.device("cpu"))
    ip = info["ipix"].numpy()
    assert ip.dtype == np.int32 and ip.min() >= 0 and ip.max() < cfg.nx * cfg.ny
    assert info["dat_calib"].shape == (8, 3001)


def test_partition_balances_uneven_tods():
    from minkasi_gb300 import parallel
    costs = [parallel.tod_cost(nd, n) for nd, n in [(256, 500000), (32, 60000), (128, 300000),
                                                    (64, 100000), (256, 200000), (32, 550000)]]
    parts = parallel.partition(costs, 2)
    assert sorted(sum(parts, [])) == list(range(6))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) / min(loads) < 1.6
    assert parallel.partition(costs, 2) == parts  # deterministic


def test_fits_image_roundtrip(tmp_path):
    """The FITS writer used by SkyMap.write / PolMap.write: 2880-byte blocks,
    80-character cards, big-endian FP64 data that reads back exactly."""
    from minkasi_gb300 import fits
    rng = np.random.default_rng(0)
    data = rng.standard_normal((7, 13))
    w6 = [200.5, 17.75, 1.0, 1.0, -2.0 / 3600, 2.0 / 3600]
    path = tmp_path / "sub" / "m.fits"
    fits.write_image(str(path), data, fits.car_header(w6))
    raw = path.read_bytes()
    assert len(raw) % 2880 == 0
    assert raw[:80].decode() == "SIMPLE  =                    T / conforms to FITS standard".ljust(80)
    back, hdr = fits.read_image(str(path))
    assert np.array_equal(back, data)
    assert (hdr["NAXIS1"], hdr["NAXIS2"]) == (13, 7)
    assert hdr["CTYPE1"] == "RA---CAR" and hdr["CTYPE2"] == "DEC--CAR"
    assert [hdr[k] for k in ("CRVAL1", "CRVAL2", "CRPIX1", "CRPIX2", "CDELT1", "CDELT2")] == w6


def test_learned_weight_files_single_and_multilevel(tmp_path):
    """A weight file holds one network (w<i>, pool) or a list of levels
    (levels, l<k>_w<i>, l<k>_pool); load gives back what save was given."""
    import torch
    from minkasi_gb300 import learned as L
    one = L.ConvNet.init(seed=0, device=torch.device("cpu"), pool=8)
    L.save(one, str(tmp_path / "one.npz"))
    b1 = L.load(str(tmp_path / "one.npz"), "cpu")
    assert isinstance(b1, L.ConvNet) and b1.pool == 8
    assert all(torch.equal(x, y) for x, y in zip(one.weights, b1.weights))
    two = [L.ConvNet.init(seed=i, device=torch.device("cpu"), pool=b) for i, b in enumerate((1, 8))]
    L.save(two, str(tmp_path / "two.npz"))
    b2 = L.load(str(tmp_path / "two.npz"), "cpu")
    assert isinstance(b2, list) and [n.pool for n in b2] == [1, 8]
    assert all(torch.equal(x, y) for a, b in zip(two, b2) for x, y in zip(a.weights, b.weights))
    # the committed weights load
    assert isinstance(L.load(L.weights_path("c1"), "cpu"), L.ConvNet)

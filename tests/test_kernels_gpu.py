"""Parity of each CUDA kernel (through the C ABI) with the oracle and with the
reference-generated golden fixtures.  GPU only."""
import numpy as np
import pytest
import torch

import oracle

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


# ---------------------------------------------------------------- projections
def test_map2tod_golden_bit_exact(K, gold):
    g = gold("proj.npz")
    for do_add, key in ((True, "map2tod_add"), (False, "map2tod_set")):
        d = dev(g["dat"])
        K.map2tod(d, dev(g["map"]), dev(g["ipix"]), do_add)
        assert np.array_equal(d.cpu().numpy(), g[key])


@pytest.mark.parametrize("n", [1, 3, 4, 5, 1000, 4099])
def test_map2tod_ragged_lengths_f32_f64(K, n):
    rng = np.random.default_rng(n)
    npix = 97
    ipix = rng.integers(0, npix, size=(1, n)).astype(np.int32)
    for dt, tdt in ((np.float64, torch.float64), (np.float32, torch.float32)):
        m = rng.standard_normal(npix).astype(dt)
        d0 = rng.standard_normal((1, n)).astype(dt)
        ref = d0.copy()
        oracle.map2tod(ref, m, ipix, True)
        d = dev(d0)
        K.map2tod(d, dev(m), dev(ipix), True)
        assert np.array_equal(d.cpu().numpy(), ref)


@pytest.mark.parametrize("maxrun", [1, 3, 6, 40, 700])
def test_map2tod_runs_across_lanes(K, maxrun):
    """Runs of equal pixels of random lengths up to maxrun (so runs cross
    the 4-sample groups of a lane, whole lanes, and the rows of 32 groups a
    warp reads), with out-of-range indices mixed in: the gathered values
    reused across lanes equal map[ipix] bit for bit, in both precisions."""
    rng = np.random.default_rng(maxrun)
    npix, n = 1000, 2 * 4096 * 4 + 37
    lens = rng.integers(1, maxrun + 1, size=n)
    pix = rng.integers(-3, npix + 3, size=n)  # a few out of range: gathered as 0
    ipix = np.repeat(pix, lens)[:n].astype(np.int32).reshape(1, n)
    for dt, tdt in ((np.float64, torch.float64), (np.float32, torch.float32)):
        m = rng.standard_normal(npix).astype(dt)
        ref = np.where((ipix >= 0) & (ipix < npix), m[np.clip(ipix, 0, npix - 1)], 0).astype(dt)
        d = torch.full((1, n), 7.0, dtype=tdt, device=cuda)
        K.map2tod(d, dev(m), dev(ipix), False)
        assert np.array_equal(d.cpu().numpy(), ref)


def test_map2tod_unaligned_view(K):
    # a view starting one element in: not 16-byte aligned -> scalar kernel
    rng = np.random.default_rng(5)
    ipix = rng.integers(0, 50, size=1001).astype(np.int32)
    m = rng.standard_normal(50)
    base = torch.zeros(1002, dtype=torch.float64, device=cuda)
    d = base[1:]
    ip = dev(np.concatenate([[0], ipix]).astype(np.int32))[1:]
    K.map2tod(d, dev(m), ip, False)
    assert np.array_equal(d.cpu().numpy(), m[ipix])


def test_tod2map_golden(K, gold):
    g = gold("proj.npz")
    m = dev(g["map"])
    K.tod2map(m, dev(g["dat"]), dev(g["ipix"]))
    assert rel(m.cpu().numpy(), g["tod2map_omp"]) < 1e-13


def test_tod2map_sorted_is_deterministic(K, gold):
    g = gold("proj.npz")
    ip = dev(g["ipix"])
    plan = K.PixPlan(ip, g["map"].size)
    outs = []
    for _ in range(2):
        m = dev(g["map"])
        plan.tod2map(m, dev(g["dat"]))
        outs.append(m.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    assert rel(outs[0], g["tod2map_omp"]) < 1e-13


def test_tod2map_large_runs_f64_f32(K):
    rng = np.random.default_rng(2)
    ndet, ndata, npix = 16, 200_003, 64 * 64
    # slowly moving pointing -> long runs of equal pixels, plus jumps
    walk = np.cumsum(rng.integers(-1, 2, size=(ndet, ndata)), axis=1) // 5
    ipix = np.mod(walk + rng.integers(0, npix, size=(ndet, 1)), npix).astype(np.int32)
    dat = rng.standard_normal((ndet, ndata))
    ref = np.zeros(npix)
    oracle.tod2map(ref, dat, ipix)
    m = torch.zeros(npix, dtype=torch.float64, device=cuda)
    K.tod2map(m, dev(dat), dev(ipix))
    assert rel(m.cpu().numpy(), ref) < 1e-12
    m32 = torch.zeros(npix, dtype=torch.float32, device=cuda)
    K.tod2map(m32, dev(dat, torch.float32), dev(ipix))
    assert rel(m32.cpu().numpy(), ref) < 2e-5
    plan = K.PixPlan(dev(ipix), npix)
    ms = torch.zeros(npix, dtype=torch.float64, device=cuda)
    plan.tod2map(ms, dev(dat))
    assert rel(ms.cpu().numpy(), ref) < 1e-12
    mt = torch.zeros(npix, dtype=torch.float64, device=cuda)
    K.tod2map_staged(mt, dev(dat), dev(ipix))
    assert rel(mt.cpu().numpy(), ref) < 1e-12


def test_tod2map_reads_pinned_host_timestream_in_place(K, gold):
    g = gold("proj.npz")
    host = torch.from_numpy(np.ascontiguousarray(g["dat"])).pin_memory()
    m = dev(g["map"])
    K.tod2map(m, host, dev(g["ipix"]))
    assert rel(m.cpu().numpy(), g["tod2map_omp"]) < 1e-13
    with pytest.raises(ValueError):
        K.tod2map(dev(g["map"]), torch.from_numpy(np.ascontiguousarray(g["dat"])), dev(g["ipix"]))


def test_tod2map_staged_golden(K, gold):
    g = gold("proj.npz")
    m = dev(g["map"])
    K.tod2map_staged(m, dev(g["dat"]), dev(g["ipix"]))
    assert rel(m.cpu().numpy(), g["tod2map_omp"]) < 1e-13
    assert K.tod2map_status() == 0


@pytest.mark.parametrize("kern", ["tod2map", "tod2map_staged"])
@pytest.mark.parametrize("n", [1, 3, 4, 5, 255, 257, 2047, 2048, 2049, 2052, 3 * 2048 * 152 + 6, 6_000_001])
def test_tod2map_ragged_sizes_and_bad_pixels(K, n, kern):
    """Warp-window and chunk edges, the <4-sample tail, more chunks than CTAs
    (6e6 samples: every staged CTA wraps its stage ring several times), runs
    that cross lanes and windows, and pixels outside [0, npix) (skipped),
    FP64 and FP32, against numpy."""
    rng = np.random.default_rng(n)
    npix = 300
    walk = np.cumsum(rng.integers(-1, 2, size=n)) // 3
    ipix = (np.mod(walk, npix + 6) - 3).astype(np.int32)  # includes -3..-1 and npix..npix+2
    dat = rng.standard_normal(n)
    ok = (ipix >= 0) & (ipix < npix)
    ref = np.zeros(npix)
    np.add.at(ref, ipix[ok], dat[ok])
    for dt, tol in ((torch.float64, 1e-12), (torch.float32, 2e-5)):
        m = torch.zeros(npix, dtype=dt, device=cuda)
        getattr(K, kern)(m, dev(dat[None, :], dt), dev(ipix[None, :]))
        assert rel(m.cpu().double().numpy(), ref) < tol, (n, dt)
    assert K.tod2map_status() == 0


@pytest.mark.parametrize("kern", ["atomic", "staged", "fixed", "sorted"])
def test_tod2map_nonfinite_samples_touch_only_their_pixels(K, kern):
    """NaN and +-inf samples: as in the reference's serial sum, a pixel is
    NaN when one of its samples is NaN or it gets both +inf and -inf, +-inf
    when it gets one sign of inf, and every other pixel is the finite sum."""
    rng = np.random.default_rng(7)
    ndet, ndata, npix = 4, 20_000, 500
    walk = np.cumsum(rng.integers(-1, 2, size=(ndet, ndata)), axis=1) // 3
    ipix = np.mod(walk + rng.integers(0, npix, size=(ndet, 1)), npix).astype(np.int32)
    dat = rng.standard_normal((ndet, ndata))
    dat[0, 100] = np.nan
    dat[1, 5000] = np.inf
    dat[3, 9000] = -np.inf
    p = ipix[2, 7000]
    j = np.flatnonzero((ipix.ravel() == p))
    j = j[j != 2 * ndata + 7000][0]
    dat[2, 7000] = np.inf
    dat.ravel()[j] = -np.inf
    ref = np.zeros(npix)
    oracle.tod2map_serial(ref, dat, ipix)
    assert np.isnan(ref).sum() >= 2 and np.isinf(ref).sum() >= 1
    m = torch.zeros(npix, dtype=torch.float64, device=cuda)
    gd, gi = dev(dat), dev(ipix)
    if kern == "atomic":
        K.tod2map(m, gd, gi)
    elif kern == "staged":
        K.tod2map_staged(m, gd, gi)
    elif kern == "fixed":
        hmax = int(np.bincount(ipix.ravel(), minlength=npix).max())
        K.tod2map_fixed(m, gd, gi, hmax, K.FixedScratch(npix, cuda))
    else:
        K.PixPlan(gi, npix).tod2map(m, gd)
    got = m.cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.array_equal(np.isposinf(got), np.isposinf(ref))
    assert np.array_equal(np.isneginf(got), np.isneginf(ref))
    fin = np.isfinite(ref)
    assert rel(got[fin], ref[fin]) < 1e-12


def test_tod2map_staged_rejects_host_and_misaligned(K, gold):
    g = gold("proj.npz")
    host = torch.from_numpy(np.ascontiguousarray(g["dat"])).pin_memory()
    with pytest.raises(ValueError):
        K.tod2map_staged(dev(g["map"]), host, dev(g["ipix"]))
    d = dev(g["dat"]).reshape(-1)
    ip = dev(g["ipix"]).reshape(-1)
    with pytest.raises(K._lib.MkError):  # 8-byte offset: not 16-byte aligned
        K.tod2map_staged(dev(g["map"]), d[1:], ip[1:])


def test_tod2map_rows_hits(K, gold):
    g = gold("solve.npz")
    hits = torch.zeros(int(g["nx"]) * int(g["ny"]), dtype=torch.float64, device=cuda)
    for k in range(int(g["ntod"])):
        K.tod2map_rows(hits, dev(g[f"t{k}_ipix"]))
    assert np.array_equal(hits.cpu().numpy().reshape(g["hits"].shape), g["hits"])


def test_check_pix_counts_out_of_range(K):
    ip = np.array([0, 5, -1, 9, 10, 3], dtype=np.int32)
    assert K.check_pix(dev(ip), 10) == 2
    with pytest.raises(Exception):
        K.PixPlan(dev(ip), 10)


# ---------------------------------------------------------------- DCT / noise
def test_dct1_golden_f64(K, gold):
    g = gold("dct.npz")
    i = 0
    while f"x{i}" in g:
        x = g[f"x{i}"]
        y = K.DCT1(x.shape[0], x.shape[1], torch.float64)(dev(x)).cpu().numpy()
        assert rel(y, g[f"y{i}"]) < 1e-13, i
        i += 1


def test_dct1_f32_and_roundtrip(K):
    x = np.random.default_rng(3).standard_normal((7, 4097))
    d = K.DCT1(7, 4097, torch.float32)
    y = d(dev(x, torch.float32))
    assert rel(y.cpu().numpy(), oracle.dct1(x)) < 2e-6
    back = d(y).cpu().numpy() / (2 * 4096)
    assert rel(back, x) < 2e-6


@pytest.mark.parametrize("fb", ["lo", "hi"])
@pytest.mark.parametrize("nrow,n", [(1, 2), (1, 3), (2, 5), (3, 13), (4, 100), (5, 331), (2, 4097),
                                    (16, 2311), (9, 694), (8, 600001), (256, 130978)])
def test_dct1_f32_four_step(K, nrow, n, fb, monkeypatch):
    """FP32 DCT-I through the four-step FFT (every 2(n-1) here factors into
    2, 3, 5, 7, 11; odd nrow leaves the last row pair half empty) against the
    FP64 oracle, with 8 and with 16 transforms per CTA ("lo", "hi")."""
    monkeypatch.setenv("MINKASI_GB300_FFT4_FB", fb)
    x = np.random.default_rng(n).standard_normal((nrow, n))
    d = K.DCT1(nrow, n, torch.float32)
    assert d.engine == 0
    y = d(dev(x, torch.float32)).cpu().numpy()
    ref = oracle.dct1(x)
    assert rel(y, ref) < 3e-6
    assert np.linalg.norm(y - ref) < 2e-6 * np.linalg.norm(ref)


@pytest.mark.parametrize("fb,passes", [("lo", "3"), ("hi", "3"), ("hi", "4")])
@pytest.mark.parametrize("nrow,n", [(3, 38), (3, 1000), (4, 700), (5, 18623), (2, 465551), (16, 144278)])
def test_dct1_f32_bluestein(K, nrow, n, fb, passes, monkeypatch):
    """Lengths whose 2(n-1) has a prime factor above 11 (37, 37, 233, 9311,
    9311, 72139): Bluestein's algorithm on the four-step passes, against the
    FP64 oracle (8 and 16 transforms per CTA; the fused middle pass and the
    four-pass form); the last two are c2 TOD lengths."""
    monkeypatch.setenv("MINKASI_GB300_FFT4_FB", fb)
    monkeypatch.setenv("MINKASI_GB300_FFT4_BLUE3", "0" if passes == "4" else "1")
    x = np.random.default_rng(n).standard_normal((nrow, n))
    d = K.DCT1(nrow, n, torch.float32)
    assert d.engine == 2
    y = d(dev(x, torch.float32)).cpu().numpy()
    ref = oracle.dct1(x)
    assert rel(y, ref) < 1e-5
    assert np.linalg.norm(y - ref) < 4e-6 * np.linalg.norm(ref)


@pytest.mark.parametrize("fb", ["lo", "hi"])
@pytest.mark.parametrize("nrow,n", [(1, 2), (3, 13), (5, 331), (2, 4097), (9, 694), (3, 1000), (5, 18623),
                                    (8, 130978), (2, 144278)])
def test_dct1_f64_four_step(K, nrow, n, fb, monkeypatch):
    """FP64 DCT-I through the four-step FFT in double precision (Bluestein's
    algorithm for 1000, 18623 and 144278), narrow and wide tiles, against the
    FP64 oracle at 1e-12, and against cuFFT's FP64 transform."""
    monkeypatch.setenv("MINKASI_GB300_FFT4_FB", fb)
    x = np.random.default_rng(n + 7).standard_normal((nrow, n))
    d = K.DCT1(nrow, n, torch.float64)
    assert d.engine in (0, 2)
    y = d(dev(x)).cpu().numpy()
    assert rel(y, oracle.dct1(x)) < 1e-12
    try:
        K.set_dct_engine(1)
        ref = K.DCT1(nrow, n, torch.float64)
        assert ref.engine == 1
        assert rel(y, ref(dev(x)).cpu().numpy()) < 1e-13
    finally:
        K.set_dct_engine(0)


def test_dct1_engines_agree_and_fall_back(K):
    x = np.random.default_rng(9).standard_normal((6, 2311))
    own = K.DCT1(6, 2311, torch.float32)(dev(x, torch.float32)).cpu().numpy()
    x2 = np.random.default_rng(10).standard_normal((3, 1000))
    try:
        K.set_dct_engine(1)
        assert K.dct_engine() == 1
        d = K.DCT1(6, 2311, torch.float32)
        assert d.engine == 1
        ref = d(dev(x, torch.float32)).cpu().numpy()
        # engine 2: the four-step FFT for smooth lengths only, cuFFT for the rest
        K.set_dct_engine(2)
        assert K.DCT1(6, 2311, torch.float32).engine == 0
        d2 = K.DCT1(3, 1000, torch.float32)
        assert d2.engine == 1
        assert rel(d2(dev(x2, torch.float32)).cpu().numpy(), oracle.dct1(x2)) < 3e-6
    finally:
        K.set_dct_engine(0)
    assert rel(own, ref) < 3e-6
    with pytest.raises(Exception):
        K.set_dct_engine(3)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_noise_plans_sharing_one_workspace(K, dtype):
    """Plans of different shapes on one workspace (as the batched operator
    builds them), used alternately: each gives what it gives on a workspace
    of its own.  Plan state (transform tables, status word) must not live in
    the shared workspace."""
    shapes = [(16, 3529), (16, 4236), (32, 4097), (16, 1000)]  # the last through Bluestein in FP32
    ws_bytes = max(K.noise_workspace_bytes(nd, n, dtype) for nd, n in shapes)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    rng = np.random.default_rng(11)
    cases = []
    for nd, n in shapes:
        A = np.linalg.qr(rng.standard_normal((nd, nd)))[0]
        cases.append((dev(A, dtype), dev(A.T, dtype), dev(rng.random((nd, n)), dtype),
                      dev(rng.standard_normal((nd, n)), dtype)))
    shared = [K.NoisePlan(nd, n, dtype, workspace=ws) for nd, n in shapes]
    alone = [K.NoisePlan(nd, n, dtype) for nd, n in shapes]
    for _ in range(2):
        for p_s, p_a, (v, vT, w, x) in zip(shared, alone, cases):
            # the tensor-core rotation (its operand image is workspace too)
            # where the shape allows it
            mode = 2 if dtype == torch.float32 and x.shape[0] in (32, 64, 128, 256) else 1
            a = p_s.apply(v, vT, w, x, rot_mode=mode)
            b = p_a.apply(v, vT, w, x, rot_mode=mode)
            assert torch.equal(a, b)
    for p_s in shared:
        assert p_s.status() == 0


def test_apply_noise_golden_f64(K, gold):
    g = gold("noise.npz")
    v, vT, w = dev(g["v"]), dev(g["vT"]), dev(g["mywt"])
    for key_x, key_dd in (("x", "dd"), ("x_short", "dd_short")):
        x = g[key_x]
        plan = K.NoisePlan(x.shape[0], x.shape[1], torch.float64)
        dd = plan.apply(v, vT, w, dev(x)).cpu().numpy()
        assert rel(dd, g[key_dd]) < 1e-12, key_x
    # in place (out aliases dat)
    x = dev(g["x"])
    plan = K.NoisePlan(x.shape[0], x.shape[1], torch.float64)
    plan.apply(v, vT, w, x, out=x)
    assert rel(x.cpu().numpy(), g["dd"]) < 1e-12


@pytest.mark.parametrize("nd,n", [(64, 70_001), (256, 140_000), (37, 1001)])
def test_sliced_fp64_rotation(K, nd, n):
    """rot_mode 4: FP64 R = A X from exact 7-bit integer slices on the bf16
    tensor cores, against numpy's FP64 product, on columns whose scales span
    1e-200 .. 1e+200 (and all-zero columns), more columns than one block
    holds, and detector counts that are not tile multiples."""
    rng = np.random.default_rng(nd)
    A = np.linalg.qr(rng.standard_normal((nd, nd)))[0]
    A[:, 3] *= 1e-9                     # entries of very different size in a row
    X = rng.standard_normal((nd, n)) * 10.0 ** rng.integers(-200, 200, size=n)[None, :]
    X[:, 5] = 0.0
    X[7, :] *= 1e-12
    want = A @ X
    plan = K.NoisePlan(nd, n, torch.float64)
    got = plan.rotate(dev(A), dev(X), rot_mode=4).cpu().numpy()
    # error per column relative to that column's scale (the scales differ by
    # 10^400, so a matrix-wide relative error would hide the small columns);
    # 2e-15 leaves room for numpy's own rounding over sums of up to 256 terms
    scale = np.abs(A).sum(axis=1)[:, None] * np.abs(X).max(axis=0)[None, :] + 1e-300
    assert np.max(np.abs(got - want) / scale) < 2e-15
    assert np.array_equal(got[:, 5], np.zeros(nd))


def test_apply_noise_golden_f64_sliced_rotation(K, gold):
    """The reference's apply_noise (noise.npz) with the sliced FP64 rotation."""
    g = gold("noise.npz")
    v, vT, w = dev(g["v"]), dev(g["vT"]), dev(g["mywt"])
    for key_x, key_dd in (("x", "dd"), ("x_short", "dd_short")):
        x = g[key_x]
        plan = K.NoisePlan(x.shape[0], x.shape[1], torch.float64)
        dd = plan.apply(v, vT, w, dev(x), rot_mode=4).cpu().numpy()
        assert rel(dd, g[key_dd]) < 1e-12, key_x


def test_apply_noise_prewhitened_by_folding(K, gold):
    g = gold("noise.npz")
    nv = g["pw_noisevec"]
    v = g["pw_v"] / nv[None, :]
    vT = g["pw_vT"] / nv[:, None]
    x = g["x"]
    plan = K.NoisePlan(x.shape[0], x.shape[1], torch.float64)
    dd = plan.apply(dev(v), dev(vT), dev(g["pw_mywt"]), dev(x)).cpu().numpy()
    assert rel(dd, g["pw_dd"]) < 1e-12


@pytest.mark.parametrize("engine,fb", [(0, "lo"), (0, "hi"), (1, "")])
def test_apply_noise_f32_close_to_f64(K, gold, engine, fb, monkeypatch):
    """FP32 apply_noise (the filter epilogue of pass B, weights staged in
    shared memory on narrow tiles that leave room for it, read directly
    otherwise) against the reference's FP64 output."""
    monkeypatch.setenv("MINKASI_GB300_FFT4_FB", fb)
    g = gold("noise.npz")
    try:
        K.set_dct_engine(engine)
        for key_x, key_dd in (("x", "dd"), ("x_short", "dd_short")):
            x = g[key_x]
            plan = K.NoisePlan(x.shape[0], x.shape[1], torch.float32)
            dd = plan.apply(dev(g["v"], torch.float32), dev(g["vT"], torch.float32),
                            dev(g["mywt"], torch.float32), dev(x, torch.float32), rot_mode=1)
            assert rel(dd.cpu().numpy(), g[key_dd]) < 1e-5, (engine, key_x, plan.engine)
            # in place
            xx = dev(x, torch.float32)
            plan.apply(dev(g["v"], torch.float32), dev(g["vT"], torch.float32),
                       dev(g["mywt"], torch.float32), xx, out=xx, rot_mode=1)
            assert torch.equal(xx, dd)
    finally:
        K.set_dct_engine(0)


# ---------------------------------------------------------------- map algebra / PCG
def test_dot_is_fp64_and_reproducible(K):
    rng = np.random.default_rng(4)
    a, b = rng.standard_normal(1_000_003), rng.standard_normal(1_000_003)
    R = K.Reducer()
    r1 = R.dot(dev(a), dev(b)).item()
    r2 = R.dot(dev(a), dev(b)).item()
    assert r1 == r2
    assert abs(r1 - float(np.dot(a, b))) < 1e-10 * np.abs(a * b).sum()
    r32 = R.dot(dev(a, torch.float32), dev(b, torch.float32)).item()
    exact32 = float(np.dot(a.astype(np.float32).astype(np.float64), b.astype(np.float32).astype(np.float64)))
    assert abs(r32 - exact32) < 1e-10 * np.abs(a * b).sum()


def test_pcg_recurrence_matches_reference(K, gold):
    g = gold("solve.npz")
    tods = [oracle.OracleTod(ipix=g[f"t{k}_ipix"], v=g[f"t{k}_v"], vT=g[f"t{k}_vT"],
                             mywt=g[f"t{k}_mywt"], dat=g[f"t{k}_dat"]) for k in range(int(g["ntod"]))]
    shape = (int(g["nx"]), int(g["ny"]))
    plans = [K.NoisePlan(t.ipix.shape[0], t.ipix.shape[1], torch.float64) for t in tods]
    dt = [(dev(t.ipix), dev(t.v), dev(t.vT), dev(t.mywt)) for t in tods]

    def A(x):
        out = torch.zeros_like(x)
        for (ip, v, vT, w), pl in zip(dt, plans):
            tmp = torch.empty(ip.shape, dtype=x.dtype, device=cuda)
            K.map2tod(tmp, x, ip, False)
            pl.apply(v, vT, w, tmp, out=tmp)
            K.tod2map(out, tmp, ip)
        return out

    ax = A(dev(g["xr"])).cpu().numpy()
    assert rel(ax, g["Axr"]) < 1e-12
    b = dev(g["rhs"])
    M = dev(g["precon"])
    x = torch.zeros_like(b)
    r, z, p = torch.empty_like(b), torch.empty_like(b), torch.empty_like(b)
    s = torch.zeros(8, dtype=torch.float64, device=cuda)
    R = K.Reducer()
    K.pcg_init(r, z, p, b, A(x), M, s, R)
    for _ in range(8):
        K.pcg_update(x, r, z, p, A(p), M, s, R)
    assert s[6].item() == 0.0 and s[7].item() == 8.0
    assert rel(x.cpu().numpy(), g["pcg8"]) < 1e-9

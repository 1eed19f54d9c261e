"""Neural radiance cache: FP64 oracle checks (CPU) and the tensor-core kernels against it (GPU).

Tolerances: the GPU keeps FP16 weights/activations with FP32 accumulation; the oracle quantises at
the same points and accumulates in FP64, so outputs agree to |d| <= 2e-2 |ref| + 2e-3 and gradients to
a relative L2 error below 3e-2 (cosine > 0.999). Gradients are loss-scaled by 128 on the GPU.
"""
import numpy as np
import pytest

LOSS_SCALE = 128.0
DIMS = [216, 64, 64, 64, 64, 64, 3]


def _split(w):
    out, o = [], 0
    for a, b in zip(DIMS[:-1], DIMS[1:]):
        out.append(w[o:o + a * b].reshape(b, a).astype(np.float64))
        o += a * b
    return out


def _encode(x):
    k = 2.0 ** np.arange(12)
    a = np.pi * x[:, :, None].astype(np.float64) * k[None, None, :]
    e = np.stack([np.sin(a), np.cos(a)], -1)  # n, 9, 12, 2
    return e.reshape(len(x), 216)


def np_forward_grad(w, x, t, den=None):
    """Unquantised FP64 MLP with the same loss (independent of the C oracle). The relative-L2
    denominator is a stop-gradient: pass `den` to hold it fixed (finite differences)."""
    Ws = _split(w)
    acts = [_encode(x)]
    for i, W in enumerate(Ws):
        z = acts[-1] @ W.T
        acts.append(np.maximum(z, 0) if i < 5 else z)
    y = acts[-1]
    if den is None:
        den = y * y + 0.01
    loss = np.mean(np.sum((y - t) ** 2 / den, 1))
    d = 2 * (y - t) / den / len(x)
    grads = []
    for i in range(5, -1, -1):
        grads.append(d.T @ acts[i])
        if i:
            d = (d @ Ws[i]) * (acts[i] > 0)
    return y, loss, np.concatenate([g.reshape(-1) for g in grads[::-1]])


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.random((n, 9)).astype(np.float32)
    x[:, 3:] = x[:, 3:] * 2 - 1
    t = (0.5 + 0.3 * np.sin(6 * x[:, :3]) * np.cos(3 * x[:, 3:6])).astype(np.float32)
    return x, t


def _weights(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    parts = []
    for a, b in zip(DIMS[:-1], DIMS[1:]):
        parts.append(rng.uniform(-1, 1, a * b) * np.sqrt(6.0 / a) * scale)
    return np.concatenate(parts).astype(np.float32)


def test_numpy_reference_gradient_finite_differences():
    x, t = _data(8, 1)
    w = _weights(2).astype(np.float64)
    y, _, g = np_forward_grad(w, x, t)
    den = y * y + 0.01
    rng = np.random.default_rng(3)
    for i in rng.choice(len(w), 12, replace=False):
        e = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += e
        wm[i] -= e
        fd = (np_forward_grad(wp, x, t, den)[1] - np_forward_grad(wm, x, t, den)[1]) / (2 * e)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])


def test_oracle_matches_unquantised_reference(orc):
    x, t = _data(256, 4)
    w = _weights(5)
    y_np, l_np, g_np = np_forward_grad(w.astype(np.float64), x, t)
    y_o = orc.nrc_forward(w, x)
    l_o, g_o = orc.nrc_grad(w, x, t)
    np.testing.assert_allclose(y_o, y_np, rtol=5e-2, atol=5e-3)
    assert abs(l_o - l_np) <= 2e-2 * l_np
    cos = g_o @ g_np / (np.linalg.norm(g_o) * np.linalg.norm(g_np))
    assert cos > 0.999


def test_oracle_adam_step(orc):
    w = _weights(6)
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    g = np.random.default_rng(7).standard_normal(len(w)).astype(np.float32)
    w0 = w.copy()
    orc.nrc_adam(w, m, v, g, 1, 1e-3)
    # first bias-corrected Adam step moves every weight by ~lr * sign(g)
    np.testing.assert_allclose(w0 - w, 1e-3 * np.sign(g), atol=2e-6)


# ---- GPU ---------------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def tracer(native_lib):
    t = native_lib.Tracer(0)
    yield t
    t.close()


def _set(tracer, w):
    from arcadia_gb300.native import lib, _p

    rc = lib().arc_nrc_set_weights(tracer.ctx, _p(np.ascontiguousarray(w, np.float32)))
    assert rc == 0, tracer.last_error()


@pytest.mark.gpu
def test_gpu_inference_matches_oracle(orc, tracer):
    import torch
    from arcadia_gb300.native import lib

    x, _ = _data(4099, 8)  # not a multiple of the 16-row tile
    w = _weights(9)
    _set(tracer, w)
    dx = torch.from_numpy(x).cuda()
    dy = torch.zeros((len(x), 3), dtype=torch.float32, device="cuda")
    assert lib().arc_nrc_query_dev(tracer.ctx, dx.data_ptr(), None, len(x), dy.data_ptr()) == 0
    tracer.synchronize()
    y = dy.cpu().numpy()
    ref = orc.nrc_forward(w, x)
    assert np.all(np.abs(y - ref) <= 2e-2 * np.abs(ref) + 2e-3), np.max(np.abs(y - ref))
    # albedo epilogue: one FP32 multiply per channel of the same network output
    alb = np.random.default_rng(3).uniform(0.1, 0.9, (len(x), 3)).astype(np.float32)
    dm = torch.zeros_like(dy)
    assert lib().arc_nrc_query_dev(tracer.ctx, dx.data_ptr(), torch.from_numpy(alb).cuda().data_ptr(), len(x),
                                   dm.data_ptr()) == 0
    tracer.synchronize()
    np.testing.assert_array_equal(dm.cpu().numpy(), y * alb)


@pytest.mark.gpu
def test_gpu_gradient_matches_oracle(orc, tracer):
    import torch
    from arcadia_gb300.native import lib

    x, t = _data(1000, 10)  # not a multiple of the 64-sample CTA tile
    w = _weights(11)
    _set(tracer, w)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    dg = torch.zeros(30400, dtype=torch.float32, device="cuda")
    assert lib().arc_nrc_grad_dev(tracer.ctx, dx.data_ptr(), dt.data_ptr(), len(x), dg.data_ptr()) == 0
    tracer.synchronize()
    g = dg.cpu().numpy().astype(np.float64) / LOSS_SCALE
    _, ref = orc.nrc_grad(w, x, t)
    cos = g @ ref / (np.linalg.norm(g) * np.linalg.norm(ref))
    rel = np.linalg.norm(g - ref) / np.linalg.norm(ref)
    assert cos > 0.999 and rel < 3e-2, (cos, rel)
    # per layer as well, so one broken layer cannot hide behind the others
    o = 0
    for a, b in zip(DIMS[:-1], DIMS[1:]):
        gl, rl = g[o:o + a * b], ref[o:o + a * b]
        assert np.linalg.norm(gl - rl) <= 5e-2 * np.linalg.norm(rl) + 1e-8, (a, b)
        o += a * b


@pytest.mark.gpu
def test_gpu_adam_step_matches_oracle(orc, tracer):
    import torch
    from arcadia_gb300.native import lib
    import ctypes

    x, t = _data(512, 12)
    w = _weights(13)
    _set(tracer, w)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    dg = torch.zeros(30400, dtype=torch.float32, device="cuda")
    assert lib().arc_nrc_grad_dev(tracer.ctx, dx.data_ptr(), dt.data_ptr(), len(x), dg.data_ptr()) == 0
    tracer.synchronize()
    g = dg.cpu().numpy() / np.float32(LOSS_SCALE)
    _set(tracer, w)  # resets the Adam state
    loss = ctypes.c_float()
    assert lib().arc_nrc_train_step_dev(tracer.ctx, dx.data_ptr(), dt.data_ptr(), len(x), 1e-3, ctypes.byref(loss)) == 0
    wg = np.zeros(30400, np.float32)
    assert lib().arc_nrc_get_weights(tracer.ctx, wg.ctypes.data) == 0
    wo, m, v = w.copy(), np.zeros_like(w), np.zeros_like(w)
    orc.nrc_adam(wo, m, v, g, 1, 1e-3)
    np.testing.assert_allclose(wg, wo, atol=1e-6)
    l_ref, _ = orc.nrc_grad(w, x, t)
    assert abs(loss.value - l_ref) <= 2e-2 * l_ref


@pytest.mark.gpu
def test_gpu_training_reduces_loss(tracer):
    import torch
    from arcadia_gb300.native import lib
    import ctypes

    x, t = _data(65536, 14)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    assert lib().arc_nrc_init(tracer.ctx, 1) == 0
    losses = []
    loss = ctypes.c_float()
    for step in range(300):
        assert lib().arc_nrc_train_step_dev(tracer.ctx, dx.data_ptr(), dt.data_ptr(), len(x), 1e-3,
                                            ctypes.byref(loss)) == 0
        losses.append(loss.value)
    assert np.isfinite(losses).all()
    assert np.mean(losses[-10:]) < 0.1 * np.mean(losses[:3]), (losses[:3], losses[-3:])


@pytest.mark.gpu
def test_gpu_weight_ema_feeds_inference(orc, tracer):
    """After each Adam step ema = d * ema + (1 - d) * w (FP32), and the query evaluates the EMA weights."""
    import torch
    from arcadia_gb300.native import lib

    x, t = _data(2048, 15)
    w = _weights(16)
    _set(tracer, w)
    d = np.float32(0.9)
    assert lib().arc_nrc_set_ema_decay(tracer.ctx, float(d)) == 0
    assert lib().arc_nrc_set_ema_warmup(tracer.ctx, 3) == 0
    try:
        dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
        ema = w.copy()
        for k in range(1, 4):  # warm-up of 3 steps: decay min(0.9, (1 + k) / (3 + k)) = 0.5, 0.6, 0.6667
            assert lib().arc_nrc_train_step_dev(tracer.ctx, dx.data_ptr(), dt.data_ptr(), len(x), 1e-3, None) == 0
            wk = np.zeros(30400, np.float32)
            assert lib().arc_nrc_get_weights(tracer.ctx, wk.ctypes.data) == 0
            dk = min(d, np.float32((1.0 + k) / (3.0 + k)))
            ema = dk * ema + (np.float32(1) - dk) * wk
        eg = np.zeros(30400, np.float32)
        assert lib().arc_nrc_get_ema_weights(tracer.ctx, eg.ctypes.data) == 0
        np.testing.assert_allclose(eg, ema, atol=1e-6)
        assert np.abs(eg - wk).max() > 1e-4  # the EMA lags the latest weights
        dy = torch.zeros((len(x), 3), dtype=torch.float32, device="cuda")
        assert lib().arc_nrc_query_dev(tracer.ctx, dx.data_ptr(), None, len(x), dy.data_ptr()) == 0
        tracer.synchronize()
        y, ref = dy.cpu().numpy(), orc.nrc_forward(eg, x)
        assert np.all(np.abs(y - ref) <= 2e-2 * np.abs(ref) + 2e-3), np.max(np.abs(y - ref))
        assert lib().arc_nrc_set_ema_decay(tracer.ctx, 1.0) != 0  # outside [0, 1)
    finally:
        assert lib().arc_nrc_set_ema_decay(tracer.ctx, 0.99) == 0
        assert lib().arc_nrc_set_ema_warmup(tracer.ctx, 0) == 0


@pytest.mark.gpu
def test_gpu_tcgen05_and_mma_sync_inference_agree(orc, tracer):
    """The tcgen05 (TMEM accumulator) kernel and the mma.sync kernel evaluate the same network; both stay
    within the FP16 tolerance of the FP64 oracle, including a ragged last tile and a compacted list."""
    import torch
    from arcadia_gb300.native import lib

    x, _ = _data(70001, 17)  # 547 tiles of 128, the last one ragged
    w = _weights(18)
    _set(tracer, w)
    dx = torch.from_numpy(x).cuda()
    outs = []
    try:
        for path in (1, 0, 2, 3):  # tcgen05 one tile group per CTA, mma.sync, four groups per CTA, automatic
            assert lib().arc_nrc_set_infer_path(tracer.ctx, path) == 0
            dy = torch.zeros((len(x), 3), dtype=torch.float32, device="cuda")
            assert lib().arc_nrc_query_dev(tracer.ctx, dx.data_ptr(), None, len(x), dy.data_ptr()) == 0
            tracer.synchronize()
            outs.append(dy.cpu().numpy())
        ref = orc.nrc_forward(w, x[:4096])
        for y in outs:
            assert np.all(np.abs(y[:4096] - ref) <= 2e-2 * np.abs(ref) + 2e-3), np.max(np.abs(y[:4096] - ref))
        assert np.max(np.abs(outs[0] - outs[1])) <= 1e-2 * np.max(np.abs(outs[1])) + 1e-3
        np.testing.assert_array_equal(outs[0], outs[2])  # the same MMAs per tile: identical bits
        np.testing.assert_array_equal(outs[0], outs[3])
        # compacted list on the tcgen05 path (four groups, then one): every third point, in reverse order
        assert lib().arc_nrc_set_infer_path(tracer.ctx, 2) == 0
        idx = np.arange(len(x) - 1, -1, -3, dtype=np.int32)
        dl = torch.from_numpy(idx).cuda()
        nd = torch.tensor([len(idx)], dtype=torch.int64, device="cuda")
        dz = torch.full((len(x), 3), -5.0, dtype=torch.float32, device="cuda")
        assert lib().arc_nrc_query_list_dev(tracer.ctx, dl.data_ptr(), nd.data_ptr(), len(x), dx.data_ptr(), None,
                                            dz.data_ptr()) == 0
        tracer.synchronize()
        z = dz.cpu().numpy()
        mask = np.zeros(len(x), bool)
        mask[idx] = True
        np.testing.assert_array_equal(z[mask], outs[0][mask])
        assert (z[~mask] == -5.0).all()
        assert lib().arc_nrc_set_infer_path(tracer.ctx, 1) == 0
        dz.fill_(-5.0)
        assert lib().arc_nrc_query_list_dev(tracer.ctx, dl.data_ptr(), nd.data_ptr(), len(x), dx.data_ptr(), None,
                                            dz.data_ptr()) == 0
        tracer.synchronize()
        np.testing.assert_array_equal(dz.cpu().numpy(), z)
        assert tracer.stats().device_status == 0
    finally:
        assert lib().arc_nrc_set_infer_path(tracer.ctx, 3) == 0


@pytest.mark.gpu
def test_gpu_tcgen05_and_mma_sync_gradients_agree(orc, tracer):
    """The tcgen05 training kernel (TMEM weight-gradient accumulators over several tiles per CTA, ragged
    last tile) and the mma.sync kernel give the same loss-scaled gradient and loss."""
    import ctypes
    import torch
    from arcadia_gb300.native import lib

    x, t = _data(40001, 19)
    w = _weights(20)
    _set(tracer, w)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    grads = []
    try:
        for path in (1, 0):
            assert lib().arc_nrc_set_train_path(tracer.ctx, path) == 0
            dg = torch.zeros(30400, dtype=torch.float32, device="cuda")
            assert lib().arc_nrc_grad_dev(tracer.ctx, dx.data_ptr(), dt.data_ptr(), len(x), dg.data_ptr()) == 0
            tracer.synchronize()
            grads.append(dg.cpu().numpy().astype(np.float64))
    finally:
        assert lib().arc_nrc_set_train_path(tracer.ctx, 1) == 0
    o = 0
    for a, b in zip(DIMS[:-1], DIMS[1:]):
        g1, g0 = grads[0][o:o + a * b], grads[1][o:o + a * b]
        assert np.linalg.norm(g1 - g0) <= 2e-2 * np.linalg.norm(g0) + 1e-6, (a, b, np.linalg.norm(g1 - g0) / np.linalg.norm(g0))
        o += a * b
    # and the first 2048 samples against the FP64 oracle
    dg = torch.zeros(30400, dtype=torch.float32, device="cuda")
    assert lib().arc_nrc_grad_dev(tracer.ctx, dx.data_ptr(), dt.data_ptr(), 2048, dg.data_ptr()) == 0
    tracer.synchronize()
    g = dg.cpu().numpy().astype(np.float64) / LOSS_SCALE
    _, ref = orc.nrc_grad(w, x[:2048], t[:2048])
    assert np.linalg.norm(g - ref) <= 3e-2 * np.linalg.norm(ref)
    assert tracer.stats().device_status == 0

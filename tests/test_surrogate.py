"""The learned surrogate: the oracle's arithmetic pinned by finite
differences and BF16 rounding, the GPU's packing, loss and backward pass
against the oracle, and a training run that shows what the network gains
over its polynomial baseline alone, with the plain-trace fallback closing the
gap in the simulated images."""

import math

import numpy as np
import pytest

from oracle import batch as OB
from oracle import surrogate as OS


def test_bf16_rounding_matches_torch():
    import torch

    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(size=10000).astype(np.float32),
                        (rng.normal(size=1000) * 1e-30).astype(np.float32),
                        np.array([1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -(1.0 + 2 ** -8)], np.float32)])
    ref = torch.from_numpy(x).to(torch.bfloat16).float().numpy()
    assert np.array_equal(OS.bf16(x), ref)


def test_quadratic_basis_order_matches_package():
    import torch

    from optika_gb300.surrogate import quadratic_basis

    u = np.random.default_rng(1).uniform(-1, 1, (50, 5))
    assert np.allclose(quadratic_basis(torch.from_numpy(u)).numpy(), OS.quadratic_basis(u))
    assert OS.quadratic_basis(u).shape[1] == 21


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(2)
    widths = (9, 12, 10, 3)
    ws = [rng.normal(size=(widths[l + 1], widths[l])) / math.sqrt(widths[l])
          for l in range(len(widths) - 1)]
    bs = [rng.normal(size=widths[l + 1]) * 0.1 for l in range(len(widths) - 1)]
    x = rng.uniform(-1, 1, (40, 9))
    t = rng.normal(size=(40, 2))
    lab = (rng.uniform(size=40) > 0.3).astype(np.float64)
    args = (t, lab, 1.0, 0.7, 1.0 / 40)

    def total(ws_, bs_):
        y, _, _ = OS.forward(x, ws_, bs_, rounding=False)
        return OS.loss(y, *args)

    y, zs, hs = OS.forward(x, ws, bs, rounding=False)
    dy = OS.loss_grad(y, *args, rounding=False)
    gw, gb = OS.backward(dy, ws, zs, hs, rounding=False)
    eps = 1e-6
    for l in range(len(ws)):
        for idx in [(0, 0), (1, 3), (widths[l + 1] - 1, widths[l] - 1)]:
            wp = [w.copy() for w in ws]
            wm = [w.copy() for w in ws]
            wp[l][idx] += eps
            wm[l][idx] -= eps
            fd = (total(wp, bs) - total(wm, bs)) / (2 * eps)
            assert abs(fd - gw[l][idx]) < 1e-7 + 1e-6 * abs(fd), (l, idx)
        j = widths[l + 1] // 2
        bp = [b.copy() for b in bs]
        bm = [b.copy() for b in bs]
        bp[l][j] += eps
        bm[l][j] -= eps
        fd = (total(ws, bp) - total(ws, bm)) / (2 * eps)
        assert abs(fd - gb[l][j]) < 1e-7 + 1e-6 * abs(fd)


def test_config_features_ranges():
    from optika_gb300 import configs
    from optika_gb300.surrogate import config_features

    _, _, params = configs.spectrograph_batch(200, seed=5)
    f = config_features(params)
    assert f.shape == (200, 4)
    assert np.abs(f[:, 0]).max() <= 1.0 + 1e-6 and np.abs(f[:, 3]).max() <= 1.0 + 1e-6


# --------------------------------------------------------------------------- GPU


def _surrogate(num_configs, seed=5, **kw):
    from optika_gb300 import configs
    from optika_gb300.surrogate import RayMapSurrogate

    systems, _, params = configs.spectrograph_batch(num_configs, seed=seed)
    sg = RayMapSurrogate(systems, params, wavelength=configs.SPEC_WAVELENGTH,
                         field_half=configs.SPEC_FIELD_HALF, pupil_half=configs.SPEC_PUPIL_HALF,
                         seed=seed, **kw)
    return sg, systems, params


@pytest.mark.gpu
def test_pack_matches_oracle(cuda):
    import torch

    from optika_gb300 import configs

    sg, systems, params = _surrogate(4)
    counts = np.array([3000, 1000, 5000, 2000])
    bt = sg.traced(counts, seed=21)
    g = torch.Generator(device="cuda").manual_seed(3)
    sg.coef.copy_(torch.randn(sg.coef.shape, device="cuda", generator=g) * 0.1)
    rows = int(counts.sum())
    bufs = {"x": torch.zeros((rows, 16), dtype=torch.bfloat16, device="cuda"),
            "aux": torch.zeros((rows, 4), device="cuda")}
    u = torch.zeros((rows, 8), device="cuda")
    xt = torch.zeros((16, rows), dtype=torch.bfloat16, device="cuda")
    sg._pack(bt, 0, rows, bufs, targets=True, u=u, xt=xt)
    torch.cuda.synchronize()
    x = bufs["x"].float().cpu().numpy()
    aux = bufs["aux"].cpu().numpy()
    uu = u.cpu().numpy()
    assert torch.equal(xt[:9], bufs["x"][:, :9].T)
    assert np.all(x[:, 9:] == 0)
    coef = sg.coef.cpu().numpy().astype(np.float64)
    cin = sg.cin.cpu().numpy()
    off = np.concatenate([[0], np.cumsum(counts)])
    px, py = bt.bufs["px"].cpu().numpy(), bt.bufs["py"].cpu().numpy()
    lab = bt.bufs["unvignetted"].cpu().numpy().astype(bool)
    for c in range(4):
        sl = slice(off[c], off[c + 1])
        gi = OB.batch_inputs(21, c, int(counts[c]), *configs.SPEC_WAVELENGTH,
                             *configs.SPEC_FIELD_HALF, configs.SPEC_PUPIL_HALF)
        uo = OS.features(gi["wavelength"], gi["field_x"], gi["field_y"], gi["pupil_x"],
                         gi["pupil_y"], *configs.SPEC_WAVELENGTH, *configs.SPEC_FIELD_HALF,
                         configs.SPEC_PUPIL_HALF)
        assert np.array_equal(uu[sl, :5], uo)
        assert np.all(uu[sl, 5] == c)
        feat = np.concatenate([uo, np.broadcast_to(cin[c], (len(uo), 4))], axis=1)
        assert np.array_equal(x[sl, :9], OS.bf16(feat))
        F = OS.quadratic_basis(uo)
        bx, by = F @ coef[c, 0], F @ coef[c, 1]
        m = lab[sl]
        s = sg.sg.out_scale
        assert np.allclose(aux[sl, 0][m], ((px[sl] - bx) / s)[m], atol=2e-4)
        assert np.allclose(aux[sl, 1][m], ((py[sl] - by) / s)[m], atol=2e-4)
        assert np.array_equal(aux[sl, 2], m.astype(np.float32))


@pytest.mark.gpu
def test_gradients_match_oracle(cuda):
    """One backward pass of the tensor-core kernels against the float64
    oracle fed the same BF16 weights and inputs (rounded where the GPU
    stores BF16)."""
    import torch

    sg, _, _ = _surrogate(4)
    bt = sg.traced(np.array([3000, 2000, 2500, 700]), seed=8)
    mlp = sg.mlp
    # non-trivial output layer so that every gradient is exercised
    g = torch.Generator(device="cuda").manual_seed(4)
    mlp.w[-1].copy_(torch.randn(mlp.w[-1].shape, device="cuda", generator=g) * 0.1)
    for b in mlp.b:
        b.copy_(torch.randn(b.shape, device="cuda", generator=g) * 0.1)
    mlp.refresh_bf16()
    sg.coef.zero_()
    sg.sg.out_scale = 5.0  # residuals of order 1 with a zero baseline
    rows = 4096
    bufs = mlp.buffers(rows, train=True)
    perm = torch.randperm(bt.total, device="cuda", generator=g)
    sg._pack(bt, 0, rows, bufs, perm=perm, targets=True, xt=bufs["xt"])
    mlp.forward(bufs, rows, train=True)
    bufs["sums"].zero_()
    lib = sg.lib
    from optika_gb300 import _lib as L
    from optika_gb300._api import ptr, stream_handle

    w_pos, w_cls, norm = 1.0, 0.5, 1.0 / rows
    L.check(lib.otx_surrogate_loss(ptr(bufs["y"]), 4, ptr(bufs["aux"]), rows, w_pos, w_cls, norm,
                                   ptr(bufs["dy"]), ptr(bufs["dyt"]), rows, ptr(bufs["sums"]),
                                   stream_handle()), "loss")
    mlp.backward(bufs, rows)
    torch.cuda.synchronize()
    mlp.check_errors()

    x = bufs["x"][:, :9].float().cpu().numpy()
    aux = bufs["aux"].cpu().numpy()
    ws = [mlp.w16[l][:, :mlp.widths[l]].float().cpu().numpy() for l in range(len(mlp.w))]
    bs = [b.cpu().numpy() for b in mlp.b]
    y, zs, hs = OS.forward(x, ws, bs)
    y_gpu = bufs["y"][:, :3].cpu().numpy()
    assert np.abs(y_gpu - y).max() < 2e-2 * (np.abs(y).max() + 1)
    # the loss from the GPU's own outputs, so that rounding-tie flips in the
    # forward pass do not leak into the gradient comparison
    dy = OS.loss_grad(y_gpu.astype(np.float64), aux[:, :2], aux[:, 2], w_pos, w_cls, norm)
    dy_gpu = bufs["dy"][:, :3].float().cpu().numpy()
    assert np.abs(dy_gpu - dy).max() <= 1e-2 * np.abs(dy).max()
    sums = bufs["sums"].cpu().numpy()
    lab = aux[:, 2]
    e = (y_gpu[:, 0] - aux[:, 0]) ** 2 + (y_gpu[:, 1] - aux[:, 1]) ** 2
    assert abs(sums[0] - np.sum(lab * e)) < 1e-3 * abs(np.sum(lab * e)) + 1e-3
    assert sums[2] == lab.sum()
    gw, gb = OS.backward(dy, ws, zs, hs)
    for l in range(len(ws)):
        gpu_w = mlp.gw[l].cpu().numpy()
        gpu_b = mlp.gb[l].cpu().numpy()
        rel_w = np.linalg.norm(gpu_w - gw[l]) / np.linalg.norm(gw[l])
        rel_b = np.linalg.norm(gpu_b - gb[l]) / np.linalg.norm(gb[l])
        assert rel_w < 2e-2 and rel_b < 2e-2, (l, rel_w, rel_b)


@pytest.mark.gpu
def test_training_gain_and_fallback_image(cuda):
    """Trained on the plain trace's rays, the network must cut the held-out
    image-position error of its quadratic baseline at least in half and
    classify vignetting; the simulated images (network + traced fallback)
    must match the plain trace's images of the same rays."""
    import torch

    sg, systems, _ = _surrogate(8)
    n_cfg = len(systems)
    train = sg.traced(np.full(n_cfg, 250_000), seed=105)
    sg.fit_baseline(train)
    hist = sg.train(train, steps=1500, batch=16384, lr=2e-3, log_every=500)
    assert hist[-1]["accuracy"] > 0.98
    held = sg.traced(np.full(n_cfg, 20_000), seed=205)
    ev = sg.evaluate(held)
    assert ev["rms_px"] < 0.5 * ev["baseline_rms_px"], ev
    assert ev["fallback_fraction"] < 0.2, ev
    assert ev["efficiency_rel_error"] < 1e-2, ev

    # image simulation against the plain trace of the same rays
    img_bt = sg.traced(np.full(n_cfg, 100_000), seed=305, image=True, outputs=())
    images, stats = sg.image(img_bt)
    sim = images.clone()
    st = stats.cpu().numpy()
    assert st[0] == img_bt.total
    assert 0 < st[1] < 0.25 * st[0]
    img_bt.run()
    torch.cuda.synchronize()
    ref = img_bt.images
    assert int(sim.sum()) == int(st[2] + st[3])
    rel_flux = abs(int(sim.sum()) - int(ref.sum())) / int(ref.sum())
    assert rel_flux < 1e-2, rel_flux
    # the images agree pixel by pixel up to rays landing one pixel over
    diff = (sim.double() - ref.double()).abs().sum().item() / ref.sum().item()
    assert diff < 0.5, diff


def _trained(num_configs=4, rays=100_000, steps=300, seed=5):
    sg, systems, params = _surrogate(num_configs, seed=seed)
    train = sg.traced(np.full(num_configs, rays), seed=seed + 36)
    sg.fit_baseline(train)
    sg.train(train, steps=steps, batch=16384, lr=2e-3, log_every=steps)
    return sg, systems


@pytest.mark.gpu
def test_fused_image_matches_layer_path(cuda):
    """The fused kernel (rays generated, network on chip, one launch plus the
    traced fallback) against the layer-by-layer path (a GEMM per layer,
    activations in HBM) on the same rays: the same network with the same
    BF16 rounding points and the same SiLU, so the routing statistics and
    the count images agree up to the few rays whose FP32 accumulation order
    flips a rounding; flux images up to atomic order as well."""
    import torch

    sg, _ = _trained()
    bt = sg.traced(np.array([70_001, 5_000, 130_007, 999]), seed=43, image=True, outputs=())
    img_a, st_a = sg.image(bt, fused=False)
    img_a, st_a = img_a.clone(), st_a.cpu().numpy()
    img_b, st_b = sg.image(bt, fused=True)
    torch.cuda.synchronize()
    sg.mlp.check_errors()
    st_b = st_b.cpu().numpy()
    n = bt.total
    assert st_a[0] == st_b[0] == n
    assert abs(int(st_a[1]) - int(st_b[1])) <= max(2, n // 10000), (st_a, st_b)
    assert abs(int(st_a[2] + st_a[3]) - int(st_b[2] + st_b[3])) <= max(2, n // 10000)
    diff = (img_a.long() - img_b.long()).abs().sum().item()
    assert diff <= max(4, n // 5000), (diff, st_a, st_b)
    assert int(img_b.sum()) == int(st_b[2] + st_b[3])


@pytest.mark.gpu
def test_fused_image_chunks_and_untrusted(cuda):
    """Calls over sub-ranges of the batch (first > 0, configurations split
    between calls) add up to the single call; an untrusted configuration is
    traced ray by ray, so its image equals the plain batched trace's."""
    import torch

    sg, _ = _trained()
    bt = sg.traced(np.array([40_000, 3_001, 52_777, 10_000]), seed=47, image=True, outputs=())
    one, st1 = sg.image(bt, fused=True)
    one, st1 = one.clone(), st1.cpu().numpy()
    many, st2 = sg.image(bt, chunk=17_000, fused=True)
    torch.cuda.synchronize()
    assert torch.equal(one, many)
    assert np.array_equal(st1, st2.cpu().numpy())
    # configuration 2 untrusted: all of its rays go to the trace
    sg.trusted.copy_(torch.tensor([1, 1, 0, 1], dtype=torch.uint8))
    img, st = sg.image(bt, fused=True)
    img = img.clone()
    bt.run()
    torch.cuda.synchronize()
    sg.mlp.check_errors()
    assert torch.equal(img[2], bt.images[2])
    assert int(st[1]) >= 52_777


@pytest.mark.gpu
def test_fused_predictions_match_layer_path(cuda):
    """Per-ray outputs of the fused kernel (prediction mode: no image, no
    queue) against the layer-by-layer path on the same rays."""
    import torch

    sg, _ = _trained()
    bt = sg.traced(np.array([20_000, 7_001, 33_333, 999]), seed=49)
    a = sg.predict(bt, fused=True)
    b = sg.predict(bt, fused=False)
    torch.cuda.synchronize()
    for k in ("px", "py"):
        d = (a[k] - b[k]).abs()
        # FP32 accumulation order may differ in the last bits; a ray whose
        # BF16 activations round differently moves by far less than a pixel
        assert float(d.max()) < 1e-3, (k, float(d.max()))
        assert float(d.mean()) < 1e-5, (k, float(d.mean()))
    assert float((a["logit"] - b["logit"]).abs().max()) < 0.05
    assert torch.equal(a["base_x"], b["base_x"]) and torch.equal(a["base_y"], b["base_y"])

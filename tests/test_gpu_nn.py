"""Warm-start network kernels (include/lbm_nn.h) against PyTorch on the CPU
in FP64 (the gradient oracle), on BF16-exact inputs and weights: tensor-core
convolution forward, input / weight / bias gradients, upsampling and its
adjoint, masked MSE, Adam, the signed-distance field, and the whole
encoder-decoder's parameter gradient."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _p(t):
    return C.c_void_p(t.data_ptr())


def _d(d):
    return (C.c_int * 3)(*d)


def _bf(a):
    """BF16-exact float64 copy (round-to-nearest through torch)."""
    return torch.as_tensor(a).to(torch.bfloat16).to(torch.float64)


def _to_torch_w(w, co, k, ci):
    return w.reshape(co, k, k, k, ci).permute(0, 4, 1, 2, 3).contiguous()


@pytest.mark.parametrize("ci,co,k,s,dims", [(16, 32, 3, 1, (8, 8, 16)), (32, 64, 3, 2, (8, 16, 8)),
                                            (64, 16, 3, 1, (4, 8, 8)), (16, 16, 1, 1, (8, 8, 8)),
                                            (64, 64, 3, 2, (8, 8, 8)), (32, 32, 3, 1, (6, 10, 7)),
                                            (16, 64, 3, 2, (5, 9, 6))])
def test_gpu_conv3d_fwd_bwd(gpu_lib, ci, co, k, s, dims):
    L = gpu_lib.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(ci * 7 + co + k + s)
    D, H, W = dims
    x = _bf(rng.normal(size=(D, H, W, ci)))
    w = _bf(rng.normal(size=(co, k ** 3, ci)) * 0.2)
    b = torch.as_tensor(rng.normal(size=co) * 0.1)
    # reference forward (pre-activation) and gradients
    xt = x.permute(3, 0, 1, 2)[None].clone().requires_grad_(True)
    wt = _to_torch_w(w, co, k, ci).requires_grad_(True)
    bt = b.clone().requires_grad_(True)
    yt = torch.nn.functional.conv3d(xt, wt, bt, stride=s, padding=k // 2)
    Do, Ho, Wo = yt.shape[2:]
    dy = _bf(rng.normal(size=(Do, Ho, Wo, co)))
    yt.backward(dy.permute(3, 0, 1, 2)[None])
    y_ref = yt.detach()[0].permute(1, 2, 3, 0)
    # device
    xd = x.to(torch.bfloat16).to(dev).reshape(-1)
    wd = w.to(torch.bfloat16).to(dev).reshape(-1)
    bd = b.to(torch.float32).to(dev)
    yd = torch.empty(Do * Ho * Wo * co, dtype=torch.bfloat16, device=dev)
    y32 = torch.empty(Do * Ho * Wo * co, dtype=torch.float32, device=dev)
    gpu_lib._check(L.lbm_nn_conv3d_fwd(_p(xd), _d(dims), ci, _p(wd), _p(bd), co, k, s, 0, _p(yd), _p(y32), None))
    dyd = dy.to(torch.bfloat16).to(dev).reshape(-1)
    dxd = torch.empty_like(xd)
    wtd = torch.empty_like(wd)
    dwd = torch.zeros(wd.numel(), dtype=torch.float32, device=dev)
    dbd = torch.zeros(co, dtype=torch.float32, device=dev)
    gpu_lib._check(L.lbm_nn_conv3d_bwd(_p(xd), _d(dims), ci, _p(wd), _p(wtd), co, k, s, _p(dyd), _p(dxd), _p(dwd),
                                       _p(dbd), None))
    torch.cuda.synchronize()
    y_got = y32.cpu().double().reshape(Do, Ho, Wo, co)
    assert torch.max(torch.abs(y_got - y_ref)) <= 1e-4 * torch.max(torch.abs(y_ref)) + 1e-6
    dx_ref = xt.grad[0].permute(1, 2, 3, 0)
    dx_got = dxd.cpu().double().reshape(D, H, W, ci)
    assert torch.max(torch.abs(dx_got - dx_ref)) <= 8e-3 * torch.max(torch.abs(dx_ref))
    dw_ref = wt.grad.permute(0, 2, 3, 4, 1).reshape(-1)
    assert torch.max(torch.abs(dwd.cpu().double() - dw_ref)) <= 1e-4 * torch.max(torch.abs(dw_ref))
    assert torch.max(torch.abs(dbd.cpu().double() - bt.grad)) <= 1e-4 * torch.max(torch.abs(bt.grad))
    # ReLU forward and backward through the stored output
    yr = torch.empty_like(yd)
    gpu_lib._check(L.lbm_nn_conv3d_fwd(_p(xd), _d(dims), ci, _p(wd), _p(bd), co, k, s, 1, _p(yr), None, None))
    g = dyd.clone()
    gpu_lib._check(L.lbm_nn_relu_bwd(_p(yr), _p(g), g.numel(), None))
    torch.cuda.synchronize()
    pos = yr.cpu().float() > 0
    assert torch.equal(g.cpu().float(), torch.where(pos, dyd.cpu().float(), torch.zeros_like(pos, dtype=torch.float)))


def test_gpu_upsample_add_mse_adam(gpu_lib):
    L = gpu_lib.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    dims, c = (2, 3, 4), 16
    x = _bf(rng.normal(size=(*dims, c)))
    xd = x.to(torch.bfloat16).to(dev).reshape(-1)
    up = torch.empty(8 * xd.numel(), dtype=torch.bfloat16, device=dev)
    gpu_lib._check(L.lbm_nn_upsample2(_p(xd), _d(dims), c, _p(up), 0, None))
    ref = x.repeat_interleave(2, 0).repeat_interleave(2, 1).repeat_interleave(2, 2)
    assert torch.equal(up.cpu().double().reshape(ref.shape), ref)
    g = _bf(rng.normal(size=ref.shape) * 0.25)
    gd = g.to(torch.bfloat16).to(dev).reshape(-1)
    back = torch.empty_like(xd)
    gpu_lib._check(L.lbm_nn_upsample2(_p(gd), _d(dims), c, _p(back), 1, None))
    ref_b = g.reshape(dims[0], 2, dims[1], 2, dims[2], 2, c).sum(dim=(1, 3, 5))
    assert torch.max(torch.abs(back.cpu().double().reshape(ref_b.shape) - ref_b)) <= 8e-3 * ref_b.abs().max()
    s = torch.empty_like(xd)
    gpu_lib._check(L.lbm_nn_add(_p(xd), _p(xd), _p(s), xd.numel(), None))
    assert torch.equal(s.cpu().double(), 2 * xd.cpu().double())
    # masked MSE over 4 of 16 channels
    nv = 50
    pred = torch.as_tensor(rng.normal(size=(nv, 16)), dtype=torch.float32)
    tgt = torch.as_tensor(rng.normal(size=(nv, 4)), dtype=torch.float32)
    mask = torch.as_tensor(rng.random(nv) < 0.6, dtype=torch.uint8)
    inv = 1.0 / (4 * int(mask.sum()))
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    dpred = torch.empty(nv * 16, dtype=torch.bfloat16, device=dev)
    pred_d, tgt_d, mask_d = pred.to(dev), tgt.to(dev), mask.to(dev)  # alive until the kernel has run
    gpu_lib._check(L.lbm_nn_mse(_p(pred_d), _p(tgt_d), _p(mask_d), nv, 16, 4, inv, _p(dpred), _p(loss), None))
    diff = (pred[:, :4] - tgt) * mask[:, None]
    assert abs(loss.item() - float((diff.double() ** 2).sum() * inv)) < 1e-5 * max(1.0, loss.item())
    dref = torch.zeros(nv, 16)
    dref[:, :4] = 2 * diff * inv
    assert torch.max(torch.abs(dpred.cpu().float().reshape(nv, 16) - dref)) <= 8e-3 * dref.abs().max()
    # Adam (bias-corrected) against its formula
    n = 1000
    w0 = torch.as_tensor(rng.normal(size=n), dtype=torch.float32)
    gr = torch.as_tensor(rng.normal(size=n), dtype=torch.float32)
    w = w0.clone().to(dev)
    m = torch.zeros(n, device=dev)
    v = torch.zeros(n, device=dev)
    wb = torch.empty(n, dtype=torch.bfloat16, device=dev)
    gr_d = gr.to(dev)
    for step in (1, 2):
        gpu_lib._check(L.lbm_nn_adam(_p(w), _p(wb), _p(gr_d), _p(m), _p(v), n, 1e-2, 0.9, 0.999, 1e-8, step, None))
    mr = 0.9 * (0.1 * gr) + 0.1 * gr
    vr = 0.999 * (0.001 * gr * gr) + 0.001 * gr * gr
    w1 = w0 - 1e-2 * (0.1 * gr / 0.1) / (torch.sqrt(0.001 * gr * gr / 0.001) + 1e-8)
    w2 = w1 - 1e-2 * (mr / (1 - 0.81)) / (torch.sqrt(vr / (1 - 0.999 ** 2)) + 1e-8)
    assert torch.allclose(w.cpu(), w2, atol=1e-5)
    assert torch.equal(wb.cpu(), w.cpu().to(torch.bfloat16))


def test_gpu_sdf_matches_brute_force(gpu_lib):
    from pv_dec_original_gb300 import warmstart as WS
    D, H, W = 24, 16, 16
    z, y, x = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    mask = (((x - 7.3) ** 2 + (y - 8.1) ** 2) < (5.0 + 1.5 * np.sin(z / 4.0)) ** 2).astype(np.uint8)
    sdf = WS.sdf_of_mask(mask).cpu().numpy().reshape(D, H, W)
    # brute force: distance to the nearest boundary voxel (fluid with a non-fluid 6-neighbour or on the box face)
    pad = np.pad(mask, 1)
    nb = np.zeros_like(mask, bool)
    for a in range(3):
        for s in (1, -1):
            sh = np.roll(pad, s, axis=a)[1:-1, 1:-1, 1:-1]
            nb |= sh == 0
    seeds = np.argwhere((mask > 0) & nb)
    pts = np.stack([z, y, x], -1).reshape(-1, 3)
    d2 = ((pts[:, None, :] - seeds[None, :, :]) ** 2).sum(-1).min(1)
    ref = np.sqrt(d2).reshape(D, H, W) + 0.5
    ref = np.where(mask > 0, ref, -ref)
    assert np.all(np.sign(sdf) == np.sign(ref))
    err = np.abs(sdf - ref)
    assert err.max() <= 1.0 and err.mean() <= 0.02


def test_gpu_network_gradient_vs_cpu_autograd(gpu_lib):
    """The whole encoder-decoder: parameter gradient of the masked MSE vs
    PyTorch FP64 autograd of the same network with the same BF16 weights."""
    from pv_dec_original_gb300 import warmstart as WS
    dims = (16, 8, 8)
    net = WS.WarmStartNet(dims, seed=3)
    rng = np.random.default_rng(11)
    n = dims[0] * dims[1] * dims[2]
    x = torch.zeros(n, WS.C_IN)
    x[:, :4] = torch.as_tensor(rng.normal(size=(n, 4)))
    xb = x.to(torch.bfloat16)
    tgt = torch.as_tensor(rng.normal(size=(n, 4)), dtype=torch.float32)
    mask = torch.as_tensor(rng.random(n) < 0.7, dtype=torch.uint8)
    inv = 1.0 / (4 * int(mask.sum()))
    dev = net.dev
    net.zero_grad()
    net.loss.zero_()
    y = net.forward(xb.to(dev).reshape(-1))
    d = net.loss_and_grad(y, tgt.to(dev).reshape(-1), mask.to(dev), inv)
    net.backward(d)
    torch.cuda.synchronize()
    # FP64 reference network
    wq = net.wb.cpu().double()
    bq = net.b.cpu().double()
    params = {}
    for name, m in net.meta.items():
        wv = wq[m["w_off"]:m["w_off"] + m["w_n"]].clone().requires_grad_(True)
        bv = bq[m["b_off"]:m["b_off"] + m["co"]].clone().requires_grad_(True)
        params[name] = (wv, bv)
    act = {"x": xb.double().reshape(*dims, WS.C_IN).permute(3, 0, 1, 2)[None]}
    for name, m in net.meta.items():
        src = m["src"]
        inp = (torch.nn.functional.interpolate(act[src[3:]], scale_factor=2, mode="nearest")
               if src.startswith("up:") else act[src])
        wv, bv = params[name]
        out = torch.nn.functional.conv3d(inp, _to_torch_w(wv, m["co"], m["ks"], m["ci"]), bv, stride=m["stride"],
                                         padding=m["ks"] // 2)
        if m["relu"]:
            out = torch.relu(out)
        if m["skip"]:
            out = out + act[m["skip"]]
        act[name] = out
    pred = act["out"][0].permute(1, 2, 3, 0).reshape(n, WS.C_OUT)[:, :4]
    loss = (((pred - tgt.double()) ** 2) * mask[:, None].double()).sum() * inv
    loss.backward()
    assert abs(net.loss.item() - loss.item()) <= 0.02 * loss.item()
    g_ref = torch.cat([params[k][0].grad for k in net.meta])
    g_got = net.gw.cpu().double()
    cos = float(torch.dot(g_ref, g_got) / (g_ref.norm() * g_got.norm()))
    rel = float((g_ref - g_got).norm() / g_ref.norm())
    assert cos > 0.999 and rel < 0.05, (cos, rel)
    gb_ref = torch.cat([params[k][1].grad for k in net.meta])
    assert float((gb_ref - net.gb.cpu().double()).norm() / gb_ref.norm()) < 0.05


def _vessel_mask(D=32, H=24, W=16):
    z, y, x = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    r = 5.0 + 1.5 * np.sin(z / 4.0)
    m = (((x - 7.3) ** 2 / 0.8 + (y - 11.1) ** 2) < r ** 2).astype(np.uint8)
    m[0] = 0
    m[-1] = 0
    return m


def test_gpu_ws_prior_matches_host(gpu_lib):
    """lbm_ws_prior: the jump-flooded in-slice distance against the exact one
    (the same tolerance as the 3D field), and the prior against its FP64
    restatement evaluated on the device's distance."""
    from helpers import poiseuille_prior, slice_distance
    from pv_dec_original_gb300 import warmstart as WS
    mask = _vessel_mask()
    U, tau = 0.025, 0.55
    pr = WS.Prior(mask, U, tau)
    dist = pr.dist.cpu().numpy().astype(np.float64).reshape(mask.shape)
    ref = slice_distance(mask)
    err = np.abs(dist - ref)
    assert np.all(dist[mask == 0] == 0.0)
    assert err.max() <= 1.0 and err.mean() <= 0.02, (err.max(), err.mean())
    drho, uz = poiseuille_prior(mask, U, tau, s=dist)
    np.testing.assert_allclose(pr.uz.cpu().numpy().reshape(mask.shape), uz, rtol=1e-5, atol=1e-6 * U)
    np.testing.assert_allclose(pr.drho.cpu().numpy().reshape(mask.shape), drho, rtol=1e-5, atol=1e-9)
    # fluid voxels in raster order
    np.testing.assert_array_equal(pr.idx.cpu().numpy(), np.flatnonzero(mask.reshape(-1)))


def test_gpu_ws_output_smooth_gather(gpu_lib):
    """Network output -> prior + correction -> masked smoothing -> per-node
    rho / u, against the FP64 host restatement."""
    from helpers import smooth_masked
    from pv_dec_original_gb300 import warmstart as WS
    mask = _vessel_mask()
    U, tau = 0.03, 0.6
    pr = WS.Prior(mask, U, tau)
    rng = np.random.default_rng(5)
    y = rng.normal(0.0, 0.3, (mask.size, WS.C_OUT)).astype(np.float32)
    rho, u = WS.prediction_to_device(torch.from_numpy(y.reshape(-1)).cuda(), pr, smooth=2)
    drho_p = pr.drho.cpu().numpy().astype(np.float64).reshape(mask.shape)
    uz_p = pr.uz.cpu().numpy().astype(np.float64).reshape(mask.shape)
    yy = y.astype(np.float64).reshape(mask.shape + (WS.C_OUT,))
    f = [drho_p + yy[..., 0] * U / WS.RHO_SCALE] + [yy[..., 1 + c] * U / WS.U_SCALE for c in range(3)]
    f[3] = f[3] + uz_p
    f = [smooth_masked(mask, v, 2) for v in f]
    fl = mask.reshape(-1) > 0
    np.testing.assert_allclose(rho.cpu().numpy(), 1.0 + f[0].reshape(-1)[fl], rtol=0, atol=1e-6)
    uu = u.cpu().numpy().reshape(-1, 3)
    for c in range(3):
        np.testing.assert_allclose(uu[:, c], f[1 + c].reshape(-1)[fl], rtol=0, atol=1e-6 * U + 1e-8)
    # the host read-back is the same data
    r2, u2 = WS.prediction_to_macro(mask, torch.from_numpy(y.reshape(-1)).cuda(), U, pr, smooth=2)
    np.testing.assert_array_equal(r2, rho.cpu().numpy())
    np.testing.assert_array_equal(u2, uu)


def test_gpu_init_from_macro_device_matches_host(gpu_lib):
    """lbm_init_from_macro_device builds the same state as lbm_init_from_macro."""
    from pv_dec_original_gb300 import warmstart as WS
    m = WS.vessel_members(1, seed=7)[0]
    s1, mask = WS.single_lattice(m, tau=0.6, precision="f32")
    s2, _ = WS.single_lattice(m, tau=0.6, precision="f32")
    x, pr = WS.features(mask, m["inlet_mean"], m["period"], tau=0.6)
    rng = np.random.default_rng(3)
    y = torch.from_numpy(rng.normal(0.0, 0.2, mask.size * WS.C_OUT).astype(np.float32)).cuda()
    rho, u = WS.prediction_to_device(y, pr)
    s1.init_from_macro(rho.cpu().numpy(), u.cpu().numpy(), True)
    s2.init_from_macro_device(rho.data_ptr(), u.data_ptr(), True, torch.cuda.current_stream().cuda_stream)
    np.testing.assert_array_equal(s1.distributions(), s2.distributions())
    s1.step(10)
    s2.step(10)
    np.testing.assert_array_equal(s1.distributions(), s2.distributions())


def test_gpu_network_forward_graph_matches_eager(gpu_lib):
    """The graph-replayed forward gives the eager forward's output bit for
    bit, for the captured input and for a new input of the same size."""
    import torch
    from pv_dec_original_gb300 import warmstart as WS
    dims = (16, 16, 32)
    net = WS.WarmStartNet(dims, seed=5)
    n = dims[0] * dims[1] * dims[2] * WS.C_IN
    g = torch.Generator(device="cuda").manual_seed(0)
    for k in range(2):
        x = (torch.rand(n, device="cuda", generator=g) * 2 - 1).to(torch.bfloat16)
        eager = net.forward(x).clone()
        graphed = net.forward_graphed(x).clone()
        torch.cuda.synchronize()
        assert torch.equal(eager, graphed), k


def test_gpu_conv_refuses_unbuilt_channel_counts(gpu_lib):
    """Channel counts other than 16, 32 and 64 are refused before any launch."""
    L = gpu_lib.load()
    dev = torch.device("cuda", 0)
    x = torch.zeros(8 * 8 * 8 * 48, dtype=torch.bfloat16, device=dev)
    w = torch.zeros(16 * 27 * 48, dtype=torch.bfloat16, device=dev)
    y = torch.zeros(8 * 8 * 8 * 16, dtype=torch.bfloat16, device=dev)
    rc = L.lbm_nn_conv3d_fwd(_p(x), _d((8, 8, 8)), 48, _p(w), None, 16, 3, 1, 0, _p(y), None, None)
    assert rc == -1  # LBM_ERR_ARG


def test_gpu_ws_features_match_reference(gpu_lib):
    """lbm_ws_features (one pass) against the same network input built from
    PyTorch element-wise operations: channels 0-3 equal; the scaled position
    and prior channels within one BF16 rounding (PyTorch divides by a
    scalar through its reciprocal); padding channels zero."""
    import torch
    from pv_dec_original_gb300 import warmstart as WS
    mask = _vessel_mask()
    x1, _ = WS.features(mask, 0.025, 3300.0, tau=0.55)
    x2, _ = WS.features_reference(mask, 0.025, 3300.0, tau=0.55)
    a = x1.float().reshape(-1, WS.C_IN).cpu()
    b = x2.float().reshape(-1, WS.C_IN).cpu()
    assert torch.equal(a[:, :4], b[:, :4])
    assert torch.all(a[:, 7:] == 0)
    d = (a[:, 4:7] - b[:, 4:7]).abs()
    assert torch.all(d <= b[:, 4:7].abs() * 2.0 ** -7 + 1e-30), float(d.max())

"""3x3x3 convolutions on the tcgen05 tensor cores (conv_tc.cu, selected by
lbm_nn_conv3d_fwd / _bwd: stride 1 on grids with D % 4, H % 16 and W % 8
== 0, stride 2 on even grids whose output has H % 16 and W % 8 == 0):
forward and input gradient against PyTorch on the CPU in FP64 on
BF16-exact inputs and weights, and against the mma.sync engine on the same
device buffers."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

AUTO, MMA_SYNC = 0, 1


def _p(t):
    return C.c_void_p(t.data_ptr())


def _d(d):
    return (C.c_int * 3)(*d)


def _bf(a):
    return torch.as_tensor(a).to(torch.bfloat16).to(torch.float64)


def _to_torch_w(w, co, ci):
    return w.reshape(co, 3, 3, 3, ci).permute(0, 4, 1, 2, 3).contiguous()


def _fwd(L, gpu_lib, engine, xd, dims, ci, wd, bd, co, relu, s=1):
    n = (dims[0] // s) * (dims[1] // s) * (dims[2] // s) * co
    yd = torch.empty(n, dtype=torch.bfloat16, device=xd.device)
    y32 = torch.empty(n, dtype=torch.float32, device=xd.device)
    gpu_lib._check(L.lbm_nn_set_conv_engine(engine))
    try:
        gpu_lib._check(L.lbm_nn_conv3d_fwd(_p(xd), _d(dims), ci, _p(wd), _p(bd) if bd is not None else None, co, 3,
                                           s, relu, _p(yd), _p(y32), None))
    finally:
        L.lbm_nn_set_conv_engine(AUTO)
    return yd, y32


def _bwd_dx(L, gpu_lib, engine, xd, dims, ci, wd, co, dyd, s=1):
    dxd = torch.empty_like(xd)
    wtd = torch.empty_like(wd)
    gpu_lib._check(L.lbm_nn_set_conv_engine(engine))
    try:
        gpu_lib._check(L.lbm_nn_conv3d_bwd(_p(xd), _d(dims), ci, _p(wd), _p(wtd), co, 3, s, _p(dyd), _p(dxd), None,
                                           None, None))
    finally:
        L.lbm_nn_set_conv_engine(AUTO)
    return dxd


@pytest.mark.parametrize("ci,co,dims,s", [(16, 16, (4, 16, 8), 1), (16, 64, (8, 16, 16), 1), (32, 32, (4, 32, 8), 1),
                                          (64, 64, (8, 16, 24), 1), (64, 16, (4, 16, 8), 1), (32, 64, (12, 32, 16), 1),
                                          (64, 32, (4, 48, 8), 1), (16, 32, (4, 32, 16), 2), (32, 64, (6, 64, 32), 2),
                                          (64, 64, (2, 32, 48), 2), (64, 16, (4, 96, 16), 2)])
def test_gpu_conv_tc_matches_fp64_and_mma_sync(gpu_lib, ci, co, dims, s):
    L = gpu_lib.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(ci * 3 + co + dims[0] + s)
    D, H, W = dims
    Do, Ho, Wo = D // s, H // s, W // s
    x = _bf(rng.normal(size=(D, H, W, ci)))
    w = _bf(rng.normal(size=(co, 27, ci)) * 0.2)
    b = torch.as_tensor(rng.normal(size=co) * 0.1)
    xt = x.permute(3, 0, 1, 2)[None].clone().requires_grad_(True)
    yt = torch.nn.functional.conv3d(xt, _to_torch_w(w, co, ci), b, stride=s, padding=1)
    assert tuple(yt.shape[2:]) == (Do, Ho, Wo)
    dy = _bf(rng.normal(size=(Do, Ho, Wo, co)))
    yt.backward(dy.permute(3, 0, 1, 2)[None])
    y_ref = yt.detach()[0].permute(1, 2, 3, 0)
    dx_ref = xt.grad[0].permute(1, 2, 3, 0)

    xd = x.to(torch.bfloat16).to(dev).reshape(-1)
    wd = w.to(torch.bfloat16).to(dev).reshape(-1)
    bd = b.to(torch.float32).to(dev)
    dyd = dy.to(torch.bfloat16).to(dev).reshape(-1)
    y_tc, y32_tc = _fwd(L, gpu_lib, AUTO, xd, dims, ci, wd, bd, co, 0, s)
    y_ms, y32_ms = _fwd(L, gpu_lib, MMA_SYNC, xd, dims, ci, wd, bd, co, 0, s)
    dx_tc = _bwd_dx(L, gpu_lib, AUTO, xd, dims, ci, wd, co, dyd, s)
    dx_ms = _bwd_dx(L, gpu_lib, MMA_SYNC, xd, dims, ci, wd, co, dyd, s)
    torch.cuda.synchronize()
    gpu_lib._check(L.lbm_nn_conv_status())

    # FP32 accumulation of BF16-exact products: relative 1e-5 of the output scale
    scale = float(y_ref.abs().max())
    got = y32_tc.cpu().double().reshape(Do, Ho, Wo, co)
    assert float((got - y_ref).abs().max()) <= 1e-5 * scale
    # the two engines differ only in summation order
    assert float((got - y32_ms.cpu().double().reshape(Do, Ho, Wo, co)).abs().max()) <= 1e-5 * scale
    # the BF16 output is the FP32 output rounded to nearest
    assert torch.equal(y_tc.cpu(), y32_tc.cpu().to(torch.bfloat16))
    # input gradient (BF16 output): within a BF16 rounding of the FP64 one
    dscale = float(dx_ref.abs().max())
    dx_got = dx_tc.cpu().double().reshape(D, H, W, ci)
    assert float((dx_got - dx_ref).abs().max()) <= 8e-3 * dscale
    assert float((dx_got - dx_ms.cpu().double().reshape(D, H, W, ci)).abs().max()) <= 8e-3 * dscale


def test_gpu_conv_tc_relu_and_no_bias(gpu_lib):
    """ReLU applied in the tensor-memory epilogue, and a NULL bias."""
    L = gpu_lib.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(9)
    dims, ci, co = (8, 32, 16), 32, 32
    x = _bf(rng.normal(size=(*dims, ci)))
    w = _bf(rng.normal(size=(co, 27, ci)) * 0.2)
    y_ref = torch.nn.functional.conv3d(x.permute(3, 0, 1, 2)[None], _to_torch_w(w, co, ci), None, padding=1)
    y_ref = torch.relu(y_ref)[0].permute(1, 2, 3, 0)
    xd = x.to(torch.bfloat16).to(dev).reshape(-1)
    wd = w.to(torch.bfloat16).to(dev).reshape(-1)
    _, y32 = _fwd(L, gpu_lib, AUTO, xd, dims, ci, wd, None, co, 1)
    torch.cuda.synchronize()
    gpu_lib._check(L.lbm_nn_conv_status())
    got = y32.cpu().double().reshape(*dims, co)
    assert float(got.min()) >= 0.0
    assert float((got - y_ref).abs().max()) <= 1e-5 * float(y_ref.abs().max())


def test_gpu_conv_engine_argument(gpu_lib):
    L = gpu_lib.load()
    assert L.lbm_nn_set_conv_engine(7) == -1  # LBM_ERR_ARG
    assert L.lbm_nn_set_conv_engine(AUTO) == 0


@pytest.mark.parametrize("ci,co,dims,s", [(16, 16, (4, 8, 16), 1), (32, 64, (2, 6, 32), 1), (64, 64, (3, 5, 16), 1),
                                          (64, 32, (2, 4, 48), 1), (16, 32, (4, 8, 32), 2), (32, 64, (6, 6, 64), 2),
                                          (64, 16, (2, 4, 32), 2), (32, 16, (5, 3, 16), 1)])
def test_gpu_conv_tc_weight_gradient(gpu_lib, ci, co, dims, s):
    """The tcgen05 weight gradient (output x extent a multiple of 16)
    against PyTorch FP64 and the mma.sync engine; dw is accumulated into."""
    L = gpu_lib.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(ci + 2 * co + dims[2] + s)
    D, H, W = dims
    x = _bf(rng.normal(size=(D, H, W, ci)))
    w = _bf(rng.normal(size=(co, 27, ci)) * 0.2)
    wt = _to_torch_w(w, co, ci).requires_grad_(True)
    yt = torch.nn.functional.conv3d(x.permute(3, 0, 1, 2)[None], wt, None, stride=s, padding=1)
    Do, Ho, Wo = yt.shape[2:]
    assert Wo % 16 == 0
    dy = _bf(rng.normal(size=(Do, Ho, Wo, co)))
    yt.backward(dy.permute(3, 0, 1, 2)[None])
    dw_ref = wt.grad.permute(0, 2, 3, 4, 1).reshape(-1)  # [co][tz][ty][tx][ci]
    xd = x.to(torch.bfloat16).to(dev).reshape(-1)
    wd = w.to(torch.bfloat16).to(dev).reshape(-1)
    dyd = dy.to(torch.bfloat16).to(dev).reshape(-1)
    out = {}
    for name, engine in (("tc", AUTO), ("ms", MMA_SYNC)):
        dwd = torch.full((wd.numel(),), 0.25, dtype=torch.float32, device=dev)
        wtd = torch.empty_like(wd)
        gpu_lib._check(L.lbm_nn_set_conv_engine(engine))
        try:
            gpu_lib._check(L.lbm_nn_conv3d_bwd(_p(xd), _d(dims), ci, _p(wd), _p(wtd), co, 3, s, _p(dyd), None,
                                               _p(dwd), None, None))
        finally:
            L.lbm_nn_set_conv_engine(AUTO)
        torch.cuda.synchronize()
        out[name] = dwd.cpu().double() - 0.25
    gpu_lib._check(L.lbm_nn_conv_status())
    scale = float(dw_ref.abs().max())
    assert float((out["tc"] - dw_ref).abs().max()) <= 1e-5 * scale + 1e-6
    assert float((out["tc"] - out["ms"]).abs().max()) <= 1e-5 * scale + 1e-6

"""Learned warm start: predict a steady rho / u field from the geometry and
the inlet, start the lattice there, and let the plain LBM finish the job.

The network is a 4-level 3D convolutional encoder-decoder (16, 32, 64, 64
channels, skip connections by addition, nearest-neighbour upsampling) on a
D x H x W grid (multiples of 8).  Input channels: signed distance to the
wall (``lbm_sdf_from_mask``), the fluid mask, the inlet mean velocity and
period; output channels: rho - 1 and u (scaled).  Every convolution,
its gradients, the loss and Adam run in this library's kernels
(``include/lbm_nn.h``: BF16 implicit GEMM on the tensor cores, FP32
accumulation); PyTorch only allocates device memory and builds input
tensors.  Training data are steady solutions of the plain LBM on seeded
stenosed tubes and bifurcations, computed as one packed ensemble.

The LBM has the last word: a warm-started lattice is run to the same
convergence criterion as a cold one (``steps_to_converge``, on FP64 lattices
so that the criterion sits far above the storage's rounding noise), so a
poor prediction costs steps, never accuracy.  The figure of merit is the
number of steps (and the wall time, prediction included) after which the
wall shear stress stays within 1% of the converged cold-start WSS
(``converge_with_history`` / ``first_within`` for the cold run,
``steps_to_wss`` for a warm one).  The reference always starts from
rest (Node.cpp:30-37); it has no counterpart to this module.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import capi

C_IN = 16   # padded input channels (sdf, mask, inlet mean, inlet period, axial position, Poiseuille prior u_z, rho)
C_OUT = 16  # padded output channels (rho - 1, ux, uy, uz)
# network targets, normalised by the inlet amplitude U (the flows are slow:
# u and rho - 1 scale with U): (rho - 1) / U * RHO_SCALE and u / U * U_SCALE
RHO_SCALE = 0.5
U_SCALE = 1.0
SDF_SCALE = 0.2
MEAN_SCALE = 30.0
PERIOD_SCALE = 1.0 / 4000.0

# (name, input, ci, co, kernel, stride, relu); "up:" inputs are upsampled x2,
# "+" names the tensor added to the layer's output (skip connection)
LAYERS = [
    ("c0a", "x", 16, 16, 3, 1, 1, None),
    ("c0b", "c0a", 16, 16, 3, 1, 1, None),
    ("d1", "c0b", 16, 32, 3, 2, 1, None),
    ("c1", "d1", 32, 32, 3, 1, 1, None),
    ("d2", "c1", 32, 64, 3, 2, 1, None),
    ("c2", "d2", 64, 64, 3, 1, 1, None),
    ("d3", "c2", 64, 64, 3, 2, 1, None),
    ("c3", "d3", 64, 64, 3, 1, 1, None),
    ("u2", "up:c3", 64, 64, 3, 1, 1, "c2"),
    ("c2u", "u2", 64, 64, 3, 1, 1, None),
    ("u1", "up:c2u", 64, 32, 3, 1, 1, "c1"),
    ("c1u", "u1", 32, 32, 3, 1, 1, None),
    ("u0", "up:c1u", 32, 16, 3, 1, 1, "c0b"),
    ("c0u", "u0", 16, 16, 3, 1, 1, None),
    ("out", "c0u", 16, 16, 1, 1, 0, None),
]


def _torch():
    import torch
    return torch


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _dims(d):
    return (C.c_int * 3)(*[int(v) for v in d])


class WarmStartNet:
    """Parameters, activations and gradients on one device; forward,
    backward and Adam through the C ABI."""

    def __init__(self, dims, device=0, seed=0):
        torch = _torch()
        self.torch = torch
        self.L = capi.load()
        self.dims = tuple(int(v) for v in dims)  # (D, H, W)
        assert all(v % 8 == 0 for v in self.dims), "grid dims must be multiples of 8"
        self.dev = torch.device("cuda", device)
        self.stream = torch.cuda.current_stream(self.dev)
        self.st = C.c_void_p(self.stream.cuda_stream)
        rng = np.random.default_rng(seed)
        # level of every tensor (0 = full grid) and its channels
        self.level = {"x": 0}
        self.chan = {"x": C_IN}
        w_off, b_off = 0, 0
        self.meta = {}
        for name, src, ci, co, ks, stride, relu, skip in LAYERS:
            lvl_in = self.level[src[3:]] - 1 if src.startswith("up:") else self.level[src]
            lvl_out = lvl_in + (1 if stride == 2 else 0)
            self.level[name] = lvl_out
            self.chan[name] = co
            taps = ks ** 3
            self.meta[name] = dict(src=src, ci=ci, co=co, ks=ks, stride=stride, relu=relu, skip=skip,
                                   lvl_in=lvl_in, lvl_out=lvl_out, w_off=w_off, w_n=co * taps * ci,
                                   b_off=b_off, taps=taps)
            w_off += co * taps * ci
            b_off += co
        self.nw, self.nb = w_off, b_off
        w = np.zeros(self.nw, np.float32)
        for name, m in self.meta.items():
            ci_real = 7 if m["src"] == "x" else m["ci"]
            co_real = 4 if name == "out" else m["co"]
            std = math.sqrt(2.0 / (m["taps"] * ci_real)) * (0.3 if name == "out" else 1.0)
            blk = np.zeros((m["co"], m["taps"], m["ci"]), np.float32)
            blk[:co_real, :, :ci_real] = rng.normal(0.0, std, (co_real, m["taps"], ci_real))
            w[m["w_off"]:m["w_off"] + m["w_n"]] = blk.reshape(-1)
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.w = torch.from_numpy(w).to(self.dev)
        self.wb = self.w.to(torch.bfloat16)
        self.b = torch.zeros(self.nb, **f32)
        self.gw = torch.zeros(self.nw, **f32)
        self.gb = torch.zeros(self.nb, **f32)
        self.mw, self.vw = torch.zeros(self.nw, **f32), torch.zeros(self.nw, **f32)
        self.mb, self.vb = torch.zeros(self.nb, **f32), torch.zeros(self.nb, **f32)
        self.wt = torch.empty(max(m["w_n"] for m in self.meta.values()), dtype=torch.bfloat16, device=self.dev)
        self.step_count = 0
        self._alloc()

    # ------------------------------------------------------------------ buffers
    def grid(self, lvl):
        return tuple(v >> lvl for v in self.dims)

    def nvox(self, lvl):
        g = self.grid(lvl)
        return g[0] * g[1] * g[2]

    def _alloc(self):
        torch = self.torch
        bf = dict(dtype=torch.bfloat16, device=self.dev)
        self.act, self.grad, self.up, self.pre = {}, {}, {}, {}
        for name, m in self.meta.items():
            n = self.nvox(m["lvl_out"]) * m["co"]
            self.act[name] = torch.empty(n, **bf)
            self.grad[name] = torch.empty(n, **bf)
            if m["src"].startswith("up:"):
                self.up[name] = torch.empty(self.nvox(m["lvl_in"]) * m["ci"], **bf)
            if m["skip"]:
                self.pre[name] = torch.empty(n, **bf)  # the layer's own (ReLU) output before the skip sum
        self.grad_up = {k: torch.empty_like(v) for k, v in self.up.items()}
        self.skip_grad = {m["skip"]: torch.empty_like(self.act[m["skip"]]) for m in self.meta.values() if m["skip"]}
        self.y32 = torch.empty(self.nvox(0) * C_OUT, dtype=torch.float32, device=self.dev)
        self.dpred = torch.empty(self.nvox(0) * C_OUT, **bf)
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.dev)

    def _check(self, rc):
        capi._check(rc)

    # ------------------------------------------------------------------ forward
    def forward(self, x):
        """x: BF16 [D*H*W*C_IN] channels-last input; returns FP32 [voxels][C_OUT]."""
        L = self.L
        self.x = x
        for name, m in self.meta.items():
            src = m["src"]
            if src.startswith("up:"):
                s = src[3:]
                self._check(L.lbm_nn_upsample2(_ptr(self.act[s]), _dims(self.grid(self.level[s])), m["ci"],
                                               _ptr(self.up[name]), 0, self.st))
                xin = self.up[name]
            else:
                xin = x if src == "x" else self.act[src]
            w = self.wb[m["w_off"]:m["w_off"] + m["w_n"]]
            b = self.b[m["b_off"]:m["b_off"] + m["co"]]
            y32 = self.y32 if name == "out" else None
            y = self.pre[name] if m["skip"] else self.act[name]
            self._check(L.lbm_nn_conv3d_fwd(_ptr(xin), _dims(self.grid(m["lvl_in"])), m["ci"], _ptr(w), _ptr(b),
                                            m["co"], m["ks"], m["stride"], m["relu"], _ptr(y), _ptr(y32), self.st))
            if m["skip"]:
                self._check(L.lbm_nn_add(_ptr(y), _ptr(self.act[m["skip"]]), _ptr(self.act[name]), y.numel(),
                                         self.st))
        return self.y32

    def forward_graphed(self, x):
        """forward() replayed from a CUDA graph: the first call for an input
        size captures the layer launches (on a side stream) with a static
        input buffer; later calls copy x into it and replay the graph on the
        current stream.  The result buffer is the same as forward()'s."""
        torch = self.torch
        if getattr(self, "_graph", None) is None or self._graph_n != x.numel():
            self._gx = torch.empty_like(x)
            self._gx.copy_(x)
            side = torch.cuda.Stream(self.dev)
            side.wait_stream(torch.cuda.current_stream(self.dev))
            graph = torch.cuda.CUDAGraph()
            st0 = self.st
            self.st = C.c_void_p(side.cuda_stream)
            try:
                with torch.cuda.graph(graph, stream=side, capture_error_mode="relaxed"):
                    self.forward(self._gx)
            finally:
                self.st = st0
            self._graph, self._graph_n = graph, x.numel()
        self._gx.copy_(x)
        self._graph.replay()
        return self.y32

    # ------------------------------------------------------------------ backward
    def backward(self, dy_out):
        """dy_out: BF16 gradient of the output layer's result; accumulates
        the parameter gradients into gw / gb."""
        L = self.L
        self.grad["out"].copy_(dy_out)
        for name in reversed(list(self.meta.keys())):
            m = self.meta[name]
            g = self.grad[name]
            if m["skip"]:
                # the sum's gradient also reaches the skip source
                self.skip_grad[m["skip"]].copy_(g)
            if m["relu"]:
                y = self.pre[name] if m["skip"] else self.act[name]
                self._check(L.lbm_nn_relu_bwd(_ptr(y), _ptr(g), g.numel(), self.st))
            src = m["src"]
            if src.startswith("up:"):
                xin, dx = self.up[name], self.grad_up[name]
            elif src == "x":
                xin, dx = self.x, None
            else:
                xin, dx = self.act[src], self.grad[src]
            w = self.wb[m["w_off"]:m["w_off"] + m["w_n"]]
            self._check(L.lbm_nn_conv3d_bwd(_ptr(xin), _dims(self.grid(m["lvl_in"])), m["ci"], _ptr(w),
                                            _ptr(self.wt), m["co"], m["ks"], m["stride"], _ptr(g), _ptr(dx),
                                            _ptr(self.gw[m["w_off"]:m["w_off"] + m["w_n"]]),
                                            _ptr(self.gb[m["b_off"]:m["b_off"] + m["co"]]), self.st))
            if src.startswith("up:"):
                s = src[3:]
                self._check(L.lbm_nn_upsample2(_ptr(dx), _dims(self.grid(self.level[s])), m["ci"],
                                               _ptr(self.grad[s]), 1, self.st))
            elif src in self.skip_grad:
                self._check(L.lbm_nn_add(_ptr(dx), _ptr(self.skip_grad[src]), _ptr(dx), dx.numel(), self.st))

    def zero_grad(self):
        self.gw.zero_()
        self.gb.zero_()

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        L = self.L
        self._check(L.lbm_nn_adam(_ptr(self.w), _ptr(self.wb), _ptr(self.gw), _ptr(self.mw), _ptr(self.vw), self.nw,
                                  lr, b1, b2, eps, self.step_count, self.st))
        self._check(L.lbm_nn_adam(_ptr(self.b), None, _ptr(self.gb), _ptr(self.mb), _ptr(self.vb), self.nb, lr, b1,
                                  b2, eps, self.step_count, self.st))

    def loss_and_grad(self, pred, target, mask, inv_norm):
        """Masked MSE over the 4 physical output channels (added to
        self.loss on the device); returns the BF16 output gradient."""
        self._check(self.L.lbm_nn_mse(_ptr(pred), _ptr(target), _ptr(mask), self.nvox(0), C_OUT, 4, inv_norm,
                                      _ptr(self.dpred), _ptr(self.loss), self.st))
        return self.dpred


# ---------------------------------------------------------------------- data
def sdf_of_mask(mask, device=0, mask_dev=None):
    """Signed distance (device FP32 [D*H*W]) of a [D][H][W] mask (mask_dev:
    the same mask already on the device, uint8, flat)."""
    torch = _torch()
    dev = torch.device("cuda", device)
    m = mask_dev if mask_dev is not None else torch.from_numpy(np.ascontiguousarray(mask, np.uint8)).to(dev)
    out = torch.empty(mask.size, dtype=torch.float32, device=dev)
    scratch = torch.empty(2 * mask.size, dtype=torch.int32, device=dev)
    st = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    capi._check(capi.load().lbm_sdf_from_mask(_ptr(m), _dims(mask.shape), _ptr(out), _ptr(scratch), st))
    return out


class Prior:
    """Device data of one vessel grid: the mask, its fluid voxels (raster
    order = the lattice's active-node order) and the slice-wise
    Hagen-Poiseuille prior (rho - 1, u_z) from ``lbm_ws_prior``."""

    def __init__(self, mask, inlet, tau, device=0, mask_dev=None):
        torch = _torch()
        self.dev = torch.device("cuda", device)
        self.shape = tuple(int(v) for v in mask.shape)
        self.n = int(mask.size)
        self.mask = (mask_dev if mask_dev is not None else
                     torch.from_numpy(np.ascontiguousarray(mask.reshape(-1), np.uint8)).to(self.dev))
        # the fluid voxels in raster order, compacted on the device
        self.idx = torch.nonzero(self.mask).reshape(-1)
        self.inlet = float(inlet)
        D = self.shape[0]
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.dist = torch.empty(self.n, **f32)
        self.drho = torch.empty(self.n, **f32)
        self.uz = torch.empty(self.n, **f32)
        scratch = torch.empty(2 * self.n + 3 * D, dtype=torch.int32, device=self.dev)
        self.stream = torch.cuda.current_stream(self.dev)
        capi._check(capi.load().lbm_ws_prior(_ptr(self.mask), _dims(self.shape), self.inlet, (tau - 0.5) / 3.0,
                                             _ptr(self.dist), _ptr(self.drho), _ptr(self.uz), _ptr(scratch),
                                             C.c_void_p(self.stream.cuda_stream)))
        self._keep = scratch

    @property
    def nact(self):
        return int(self.idx.numel())


def features(mask, inlet_mean, period, tau=0.8, device=0):
    """BF16 channels-last network input [D*H*W*C_IN] and the Prior the
    network's output corrects, built on the device in one pass
    (``lbm_ws_features``; ``features_reference`` is the same input from
    PyTorch element-wise operations)."""
    torch = _torch()
    dev = torch.device("cuda", device)
    m = torch.from_numpy(np.ascontiguousarray(mask.reshape(-1), np.uint8)).to(dev)  # one upload of the mask
    prior = Prior(mask, inlet_mean, tau, device, mask_dev=m)
    sdf = sdf_of_mask(mask, device, mask_dev=m)
    x = torch.empty(mask.size * C_IN, dtype=torch.bfloat16, device=dev)
    capi._check(capi.load().lbm_ws_features(_ptr(sdf), _ptr(prior.mask), _ptr(prior.uz), _ptr(prior.drho),
                                            _dims(mask.shape), SDF_SCALE, inlet_mean * MEAN_SCALE,
                                            period * PERIOD_SCALE, inlet_mean, RHO_SCALE, _ptr(x),
                                            C.c_void_p(prior.stream.cuda_stream)))
    return x, prior


def features_reference(mask, inlet_mean, period, tau=0.8, device=0):
    """features() from PyTorch element-wise operations (the test oracle of
    lbm_ws_features)."""
    torch = _torch()
    dev = torch.device("cuda", device)
    n = mask.size
    sdf = sdf_of_mask(mask, device)
    prior = Prior(mask, inlet_mean, tau, device)
    x = torch.zeros((n, C_IN), dtype=torch.float32, device=dev)
    x[:, 0] = torch.clamp(sdf * SDF_SCALE, -3.0, 3.0)
    x[:, 1] = prior.mask.to(torch.float32)
    x[:, 2] = inlet_mean * MEAN_SCALE
    x[:, 3] = period * PERIOD_SCALE
    # axial position (flow along z): the pressure level depends on the
    # distance to the outlet, beyond the convolutions' receptive field
    D, H, W = mask.shape
    x[:, 4] = (torch.arange(D, device=dev, dtype=torch.float32) / D).repeat_interleave(H * W)
    x[:, 5] = prior.uz / inlet_mean
    x[:, 6] = prior.drho / inlet_mean * RHO_SCALE
    return x.to(torch.bfloat16).reshape(-1).contiguous(), prior


def make_target(mask, rho, u, inlet, prior, device=0):
    """FP32 [D*H*W][4] target: the scaled correction of the prior (rho, u
    per active node, host arrays)."""
    torch = _torch()
    t = torch.zeros((mask.size, 4), dtype=torch.float32, device=prior.dev)
    r = torch.from_numpy(np.ascontiguousarray(rho, np.float64) - 1.0).to(prior.dev, torch.float32)
    uu = torch.from_numpy(np.ascontiguousarray(u, np.float32).reshape(-1, 3)).to(prior.dev)
    i = prior.idx
    t[i, 0] = (r - prior.drho[i]) / inlet * RHO_SCALE
    t[i, 1:] = uu / inlet * U_SCALE
    t[i, 3] -= prior.uz[i] / inlet * U_SCALE
    return t.reshape(-1)


def prediction_to_device(y32, prior, smooth=1):
    """Per-active-node rho (nact) and u (3 * nact, interleaved) as device
    FP32 tensors from the network output y32 ([voxels][C_OUT] FP32 on the
    device): prior + correction, smoothed over the fluid (`smooth` rounds of
    the masked [1, 2, 1] filter: one round measured best -- none leaves
    voxel-scale content that costs a bifurcation's prior thousands of steps,
    two blur the near-wall profile), gathered (``lbm_ws_output``,
    ``lbm_ws_smooth``, ``lbm_ws_gather``)."""
    torch = _torch()
    L = capi.load()
    st = C.c_void_p(prior.stream.cuda_stream)
    n, m = prior.n, prior.nact
    f32 = dict(dtype=torch.float32, device=prior.dev)
    fields = torch.empty(4 * n, **f32)
    capi._check(L.lbm_ws_output(_ptr(y32), C_OUT, _ptr(prior.mask), _ptr(prior.drho), _ptr(prior.uz), n,
                                prior.inlet, RHO_SCALE, U_SCALE, _ptr(fields), st))
    if smooth:
        tmp = torch.empty(n, **f32)
        for k in range(4):
            capi._check(L.lbm_ws_smooth(_ptr(prior.mask), _dims(prior.shape), C.c_void_p(fields.data_ptr() + 4 * k * n),
                                        _ptr(tmp), int(smooth), st))
    rho = torch.empty(m, **f32)
    u = torch.empty(3 * m, **f32)
    capi._check(L.lbm_ws_gather(_ptr(fields), n, _ptr(prior.idx), m, _ptr(rho), _ptr(u), st))
    return rho, u


def prediction_to_macro(mask, y32, inlet, prior, smooth=1):
    """prediction_to_device read back to the host: rho (nact) and u
    (nact, 3), FP32."""
    rho, u = prediction_to_device(y32, prior, smooth)
    return rho.cpu().numpy(), u.cpu().numpy().reshape(-1, 3)


def zero_output(prior):
    """A zero network output: prediction_to_device of it is the prior alone."""
    torch = _torch()
    return torch.zeros(prior.n * C_OUT, dtype=torch.float32, device=prior.dev)


def vessel_members(n, seed, box=(32, 32, 64), bifurcation_every=4, radius=(4.0, 9.0), period=(2000.0, 6000.0)):
    """Seeded stenosed tubes (and every k-th a small Y-bifurcation) filling
    a fixed box (x, y, z) between an inlet at z = 0 and an outlet at z = top,
    each with its own inlet waveform (mean 0.01-0.04, period drawn from
    `period` steps).  Tube radii are drawn from `radius` (lattice units at a
    box width of 32, scaled with the width); bifurcation parents from its
    lower end to 0.7 of the way up."""
    from . import geometry as G
    rng = np.random.default_rng(seed)
    nx, ny, nz = box
    sc = nx / 32.0
    out = []
    for m in range(n):
        mean = float(rng.uniform(0.01, 0.04))
        per = float(rng.uniform(*period))
        cx, cy = 0.5 * (nx - 1) + 0.173, 0.5 * (ny - 1) + 0.061
        if bifurcation_every and m % bifurcation_every == bifurcation_every - 1:
            r = float(rng.uniform(radius[0], radius[0] + 0.3 * (radius[1] - radius[0]))) * sc
            s = G.y_bifurcation(r, 0.72 * r, float(rng.uniform(8.0, 14.0)), z_in=1.3, z_out=nz - 1.4,
                                z_split=0.5 * nz, center=(cx, cy), seed=seed * 1000 + m, h=1.0)
            kind = "bifurcation"
        else:
            r = float(rng.uniform(*radius)) * sc
            s = G.stenosed_tube(r, nz - 2.7, float(rng.uniform(0.2, 0.7)), float(rng.uniform(0.0, 0.3)),
                                center=(cx, cy), z0=1.3, seed=seed * 1000 + m, h=max(1.0, r / 8.0))
            kind = "stenosed_tube"
        lo, hi = s.v.reshape(-1, 3).min(0), s.v.reshape(-1, 3).max(0)
        if lo.min() < 0.0 or hi[0] > nx - 1.0 or hi[1] > ny - 1.0 or hi[2] > nz:
            raise ValueError(f"member {m} leaves the {box} box")
        meta = dict(s.meta)
        s = G.add_bbox_anchors(s, (0.0, 0.0, 0.0), (nx - 1.0, ny - 1.0, float(nz)))
        s.meta = meta
        out.append({"surface": s, "radius": r, "center": (cx, cy), "inlet_mean": mean, "period": per,
                    "kind": kind})
    return out


def steady_ensemble(members, tau=0.8, steps=40000, precision="f32", device=0, collision=0):
    """Steady solutions (constant inlet at each member's mean) of all members
    advanced as one packed lattice; returns per member (mask, rho, u)."""
    from .ensemble import Ensemble
    ens = Ensemble(members, 19, precision, tau, device=device, steady=True, collision=collision)
    ens.solver.set_graph_steps(32)
    ens.step(steps)
    rho, u, mem = ens.macro()
    out = []
    for k, m in enumerate(members):
        mask = ens.member_mask(k)
        out.append((mask, rho[mem == k], u[mem == k]))
    ens.solver.close()
    return out


def residual_runner(solver, check=100):
    """Relative change of u over `check` steps, for a convergence loop."""
    prev = solver.macro()[1]

    def step():
        nonlocal prev
        solver.step(check)
        u = solver.macro()[1]
        r = float(np.max(np.abs(u - prev)) / max(np.max(np.abs(u)), 1e-30))
        prev = u
        return r

    return step


def steps_to_converge(solver, tol=1e-6, check=100, max_steps=60000):
    """Steps until max|u(t) - u(t - check)| / max|u| < tol (or max_steps);
    returns (steps, last residual)."""
    step = residual_runner(solver, check)
    n, r = 0, float("inf")
    while n < max_steps:
        r = step()
        n += check
        if r < tol:
            break
    return n, r


def converge_with_history(solver, tol=1e-6, check=100, max_steps=60000):
    """steps_to_converge that also keeps the wall shear stress after every
    `check` steps; returns (steps, last residual, [(step, wss)])."""
    step = residual_runner(solver, check)
    n, r, hist = 0, float("inf"), []
    while n < max_steps:
        r = step()
        n += check
        hist.append((n, solver.wss()["wss"].copy()))
        if r < tol:
            break
    return n, r, hist


def wss_error(w, ref):
    return float(np.linalg.norm(w - ref) / max(np.linalg.norm(ref), 1e-300))


def first_within(hist, ref, tol=0.01):
    """First step of a (step, wss) history from which the WSS error against
    `ref` stays below `tol` (None if it never settles there)."""
    ok = None
    for n, w in hist:
        if wss_error(w, ref) < tol:
            ok = n if ok is None else ok
        else:
            ok = None
    return ok


def steps_to_wss(solver, ref, tol=0.01, check=100, max_steps=60000, hold=3):
    """Steps until the WSS error against `ref` is below `tol` at `hold`
    consecutive checks (the first of them counts); None if not reached."""
    n, run = 0, 0
    while n < max_steps:
        if wss_error(solver.wss()["wss"], ref) < tol:
            run += 1
            if run == hold:
                return n - (hold - 1) * check
        else:
            run = 0
        solver.step(check)
        n += check
    return None


def single_lattice(member, tau=0.8, precision="f64", device=0, collision=0):
    """One member as its own lattice with a constant inlet (steady problem)."""
    tri = member["surface"].tri12()
    mask, vd = capi.voxelize(tri, 1.0)
    bb = np.array(vd.bbox[:])
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    s = capi.Solver(19, precision, capi.LBM_PHYSICS, tau, 1.0, (bb[0], bb[2], bb[4]), 1.0, 1.0, device,
                    collision=collision)
    s.set_geometry(mask, [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, member["center"][0],
                                       member["center"][1], member["radius"]),
                          capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)])
    s.set_normals(tri)
    s.set_inlet_table([member["inlet_mean"]])
    return s, mask


def pulsatile_lattice(member, tau=0.55, precision="f32", device=0, collision=0, check=100):
    """One member as its own lattice driven by its own waveform
    u(s) = mean (1 + 0.5 sin(2 pi s / T) + 0.2 sin(4 pi s / T)), T = its
    period rounded to a multiple of `check` steps; step 0 is phase 0, where
    the inlet is at its mean (the Poiseuille prior's amplitude).  Returns
    (solver, mask, T)."""
    from . import waveform
    T = int(check * max(1, round(member["period"] / check)))
    s, mask = single_lattice(member, tau, precision, device, collision)
    s.set_inlet_table(waveform.sinusoid_table(member["inlet_mean"], T))
    return s, mask, T


def run_periods(solver, T, check=100, tol=1e-3, max_periods=30, min_periods=2, keep=True):
    """Steps a pulsatile lattice period by period, reading the wall shear
    stress after every `check` steps, until the cycle-to-cycle change -- the
    largest over the phases of |w_k(phase) - w_k-1(phase)| / |w_k-1(phase)|
    -- is below `tol` (the converged periodic state) or max_periods have
    run.  The lattice then stands at phase 0.  Returns (history [(step,
    wss)] -- every check if `keep`, else the last two periods --, periods
    run, last change)."""
    nph = T // check
    hist, change, k = [], float("inf"), 0
    n0 = solver.counts()["steps"]
    for k in range(1, max_periods + 1):
        for _ in range(nph):
            solver.step(check)
            hist.append((solver.counts()["steps"] - n0, solver.wss()["wss"].astype(np.float32)))
        if not keep and len(hist) > 2 * nph:
            del hist[:len(hist) - 2 * nph]
        if k >= 2:
            change = max(wss_error(hist[-nph + j][1], hist[-2 * nph + j][1]) for j in range(nph))
            if change < tol and k >= min_periods:
                break
    return hist, k, change


def first_within_periodic(hist, ref_cycle, T, check=100, tol=0.01):
    """First step of a (step, wss) history from which the WSS stays within
    `tol` of the converged cycle's WSS at the same phase (ref_cycle: the
    wss of one period, one entry per check, the first after `check` steps
    of it); None if it never settles there."""
    nph = T // check
    ok = None
    for n, w in hist:
        if wss_error(w, ref_cycle[(n // check - 1) % nph]) < tol:
            ok = n if ok is None else ok
        else:
            ok = None
    return ok


def periodic_solutions(members, tau=0.55, precision="f32", device=0, collision=0, check=100, tol=1e-3,
                       max_periods=30):
    """The converged periodic state at phase 0 of every member (each on its
    own lattice from rest, run_periods): per member (mask, rho, u, period T
    in steps, periods run, last cycle-to-cycle change)."""
    out = []
    for m in members:
        s, mask, T = pulsatile_lattice(m, tau, precision, device, collision, check)
        s.set_graph_steps(check)
        _, k, ch = run_periods(s, T, check, tol, max_periods, keep=False)
        rho, u = s.macro()
        s.close()
        out.append((mask, rho, u, T, k, ch))
    return out


def periodic_arms(net, member, tau=0.55, device=0, collision=0, check=100, tol=1e-3, max_periods=30,
                  wss_tol=0.01):
    """One held-out member's pulsatile lattice (FP32) started three ways --
    from rest (cold, as the reference always starts), from the Poiseuille
    prior alone, and from the network's prediction (prior + learned
    correction) -- each run to its converged periodic state (run_periods).
    The cold run's last period is the reference.  Per arm: the first step
    from which the WSS stays within wss_tol of the reference at the same
    phase, the periods run, the prediction time (features, network forward
    replayed from its CUDA graph, prior, smoothing and state build, all on
    the device; the caller captures the graph first) and the wall time =
    prediction + steps x the lattice's measured time per step."""
    import time
    torch = _torch()
    dev = torch.device("cuda", device)
    sc, mask, T = pulsatile_lattice(member, tau, "f32", device, collision, check)
    sc.set_graph_steps(check)
    hist, kc, chc = run_periods(sc, T, check, tol, max_periods)
    nph = T // check
    ref = [w for _, w in hist[-nph:]]
    c1 = first_within_periodic(hist, ref, T, check, wss_tol)
    _, uc = sc.macro()
    sc.step(check)
    sc.sync()
    t0 = time.perf_counter()
    sc.step(10 * check)
    sc.sync()
    t_step = (time.perf_counter() - t0) / (10 * check)
    sc.close()
    row = {"kind": member["kind"], "radius": member["radius"], "period": T, "inlet_mean": member["inlet_mean"],
           "active": int(mask.sum()), "f32_us_per_step": t_step * 1e6,
           "cold": {"steps_1pct_wss": c1, "periods_run": kc, "last_cycle_change": chc,
                    "s_1pct_wss": None if c1 is None else c1 * t_step}}
    for arm in ("prior", "net"):
        sw, _, _ = pulsatile_lattice(member, tau, "f32", device, collision, check)
        sw.set_graph_steps(check)
        sw.sync()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        x, prior = features(mask, member["inlet_mean"], T, tau=tau, device=device)
        y = net.forward_graphed(x) if arm == "net" else zero_output(prior)
        rho, u = prediction_to_device(y, prior)
        sw.init_from_macro_device(rho.data_ptr(), u.data_ptr(), True, torch.cuda.current_stream(dev).cuda_stream)
        sw.sync()
        t_pred = time.perf_counter() - t0
        ua = u.cpu().numpy().reshape(-1, 3)
        hw, kw, chw = run_periods(sw, T, check, tol, kc + 1)
        w1 = first_within_periodic(hw, ref, T, check, wss_tol)
        sw.close()
        row[arm] = {"steps_1pct_wss": w1, "periods_run": kw, "last_cycle_change": chw, "predict_s": t_pred,
                    "s_1pct_wss": None if w1 is None else t_pred + w1 * t_step,
                    "err_u_phase0": float(np.linalg.norm(ua - uc) / np.linalg.norm(uc))}
    return row


def make_sample(mask, member, rho, u, tau=0.8, device=0):
    """(input, target, device mask, 1 / (4 * fluid voxels)) for training."""
    x, prior = features(mask, member["inlet_mean"], member["period"], tau, device)
    t = make_target(mask, rho, u, member["inlet_mean"], prior, device)
    return x, t, prior.mask, 1.0 / (4.0 * max(1, int(mask.sum())))


def train(net, samples, iters=400, lr=2e-3, batch=4, log=None):
    """samples: list of make_sample tuples; Adam with a cosine-decayed
    learning rate.  Returns the loss history (mean over each batch)."""
    hist = []
    rng = np.random.default_rng(0)
    base = lr
    for it in range(iters):
        lr = base * 0.5 * (1.0 + math.cos(math.pi * it / iters)) + 0.02 * base
        net.zero_grad()
        net.loss.zero_()
        for k in rng.choice(len(samples), size=min(batch, len(samples)), replace=False):
            x, t, m, inv = samples[k]
            y = net.forward(x)
            d = net.loss_and_grad(y, t, m, inv)
            net.backward(d)
        net.adam(lr)
        if it % 20 == 0 or it == iters - 1:
            hist.append(float(net.loss.item()) / batch)
            if log:
                log(it, hist[-1])
    return hist

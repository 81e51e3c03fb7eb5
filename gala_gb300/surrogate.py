"""A learned surrogate for an expensive potential (SCF), trained on the GPU.

Model (see gala_gb300/csrc/gx_mlp.cuh): an MLP y(xh) with 3 -> 256 -> 256 ->
256 -> 256 -> 1 units and SiLU activations, where xh maps the position into the
unit ball with a logarithmic radius, and

    Phi(x) = Phi_0(r) + Phi_H(r) y(xh),    Phi_H = -G M / (r + r_s),

Phi_0 being the spherical (l = 0) part of the SCF expansion, evaluated exactly,
and Phi_H a fixed radial scale, so the network only learns the bounded
non-spherical part.  Training data are (x, Phi, grad Phi) samples of
the analytic SCF potential, computed on the GPU in FP64
(gx_potential_value / gx_potential_gradient), with r log-uniform in
[r_min, r_max] and isotropic directions.  Training runs the library's own FP32
forward / backward / double-backward kernels (gx_mlp_train_step) with Adam
(gx_mlp_adam) on a loss that fits both y and dy/dxh.  Inference
(gx_surrogate_gradient, gx_surrogate_leapfrog) uses BF16 weights on the tensor
cores with FP32 accumulation (activations as BF16 hi + lo pairs by default);
the last part of training uses BF16-rounded weights in the forward pass, so the
network that is trained is the one the tensor cores evaluate.  Outside
[r_min, r_max] the analytic SCF force (FP32) is used instead.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi
from ._trace import traced
from .units import G as G_GALACTIC

H = 256
OFF_W1, OFF_B1 = 0, 768
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * H
OFF_W4 = OFF_B3 + H
OFF_B4 = OFF_W4 + H * H
OFF_W5 = OFF_B4 + H
OFF_B5 = OFF_W5 + H
NPARAM = OFF_B5 + 1
RHO0 = 0.1


def init_params(seed=0, w1_scale=3.0):
    """Kaiming-normal weights (first layer widened by `w1_scale`), zero biases,
    small output layer."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)
    p[OFF_W1:OFF_B1] = rng.normal(0, w1_scale * math.sqrt(2.0 / 3), H * 3)
    p[OFF_B1:OFF_W2] = rng.uniform(-1, 1, H)
    for off in (OFF_W2, OFF_W3, OFF_W4):
        p[off:off + H * H] = rng.normal(0, math.sqrt(2.0 / H), H * H)
    p[OFF_W5:OFF_B5] = rng.normal(0, 0.1 * math.sqrt(1.0 / H), H)
    return p


def input_map(x, r_min, r_max, xp=np):
    """xh = rho(r) x / r with rho = rho0 + (1 - rho0) ln(r / r_min) / ln(r_max / r_min)."""
    r = xp.sqrt((x ** 2).sum(axis=0))
    n = x / r
    L = math.log(r_max / r_min)
    rho = RHO0 + (1 - RHO0) * xp.log(r / r_min) / L
    drho = (1 - RHO0) / (r * L)
    return rho * n, r, n, rho, drho


def scf_l0(scf, r, xp=np):
    """Spherical part of the SCF expansion: Phi_0(r) and dPhi_0/dr (FP64),
    from phi_nl / dphi_nl at l = 0 (gala: src/gala/potential/scf/src/bfe_helper.cpp:24-64)."""
    p = scf.packed().params
    GM, rs = p[0] * p[3], p[4]
    nmax, lmax = int(p[1]), int(p[2])
    Sn = p[5:5 + (nmax + 1) * (lmax + 1) ** 2].reshape(nmax + 1, lmax + 1, lmax + 1)[:, 0, 0]
    s = r / rs
    xi = (s - 1) / (s + 1)
    i1 = 1.0 / (1.0 + s)
    C, Cm1 = xp.ones_like(s), xp.zeros_like(s)
    D, Dm1 = xp.ones_like(s), xp.zeros_like(s)
    sp = Sn[0] * C
    sd = Sn[0] * i1
    for n in range(1, nmax + 1):
        if n == 1:
            Cm1, C = C, 3.0 * xi
        else:
            Cm1, C = C, (2 * xi * (n + 0.5) * C - (n + 1.0) * Cm1) / n
        nd = n - 1
        if nd == 1:
            Dm1, D = D, 5.0 * xi
        elif nd > 1:
            Dm1, D = D, (2 * xi * (nd + 1.5) * D - (nd + 3.0) * Dm1) / nd
        sp = sp + Sn[n] * C
        sd = sd + Sn[n] * i1 * ((1 + s) * C - 6.0 * D) * i1
    return -GM / rs * sp * i1, GM / rs ** 2 * sd * i1


def truncated_scf(scf, L):
    """The SCF potential with its expansion cut at degree l <= L (the same n
    range): the analytic method at a chosen lower accuracy, the baseline a
    surrogate of the same accuracy is compared with."""
    from .potential import SCFPotential

    S, T = scf.parameters["Snlm"], scf.parameters["Tnlm"]
    return SCFPotential(m=scf.parameters["m"], r_s=scf.parameters["r_s"], Snlm=np.asarray(S)[:, :L + 1, :L + 1],
                        Tnlm=np.asarray(T)[:, :L + 1, :L + 1])


class SurrogatePotential:
    """Surrogate of an SCFPotential (or any potential whose monopole is the
    Hernquist sphere (m, r_s)), trained on the GPU."""

    def __init__(self, scf, r_min=0.5, r_max=200.0, seed=0, split=3):
        import torch

        from ._device import require_cuda

        self.dev = require_cuda()
        self.scf = scf
        if getattr(scf, "nmax", 0) + 1 > 24 or getattr(scf, "lmax", 0) + 1 > 16:
            raise ValueError("the FP32 SCF fallback supports nmax <= 23 and lmax <= 15")
        if not 0 < r_min < r_max:
            raise ValueError("need 0 < r_min < r_max")
        self.r_min, self.r_max = float(r_min), float(r_max)
        self.GM = G_GALACTIC * float(scf.parameters["m"])
        self.r_s = float(scf.parameters["r_s"])
        self.params = torch.from_numpy(init_params(seed)).to(self.dev)
        self.scf_f32 = torch.from_numpy(scf.packed().params.astype(np.float32)).to(self.dev)
        self.wbf16 = None
        self.wimg = None
        self.engine = "tcgen05"
        self.split = int(split)
        self.history = []

    # --------------------------------------------------------------- data
    def targets(self, x):
        """Features and normalised targets at positions x (3, N) float64 CUDA tensor."""
        import torch

        from ._device import ptr, stream_handle

        n = x.shape[1]
        phi = torch.empty(n, dtype=torch.float64, device=self.dev)
        grad = torch.empty((3, n), dtype=torch.float64, device=self.dev)
        desc = self.scf.packed().for_device()
        _abi.call("gx_potential_value", desc, 0.0, ptr(x), n, ptr(phi), stream_handle())
        _abi.call("gx_potential_gradient", desc, 0.0, ptr(x), n, ptr(grad), stream_handle())
        xh, r, nvec, rho, drho = input_map(x, self.r_min, self.r_max, xp=torch)
        phiH = -self.GM / (r + self.r_s)
        dphiH = self.GM / (r + self.r_s) ** 2          # d Phi_H / dr
        phi0, dphi0 = scf_l0(self.scf, r, xp=torch)
        ystar = (phi - phi0) / phiH
        v = (grad - (dphi0 + dphiH * ystar) * nvec) / phiH  # grad_x y*
        nv = (nvec * v).sum(axis=0)
        gstar = (r / rho) * (v - nvec * nv) + nvec * nv / drho  # J^-T v
        # weight of the gradient term: the physical force error is
        # |Phi_H J^T dG| ~ |grad Phi| rho (1 + r_s / r) |dG|, so weight by that factor squared
        wg = (rho * (1.0 + self.r_s / r)) ** 2
        return xh, ystar, gstar, wg

    def sample_positions(self, n, seed):
        import torch

        g = torch.Generator(device=self.dev)
        g.manual_seed(seed)
        lr = math.log(self.r_min) + torch.rand(n, generator=g, device=self.dev, dtype=torch.float64) * math.log(
            self.r_max / self.r_min)
        d = torch.randn((3, n), generator=g, device=self.dev, dtype=torch.float64)
        d = d / torch.linalg.norm(d, dim=0)
        # keep away from the z axis, where gala's SCF gradient divides by sin(theta)
        d[0] = torch.where(d[0].abs() < 1e-4, torch.full_like(d[0], 1e-4), d[0])
        return d * torch.exp(lr)

    def make_dataset(self, n_samples=16 * 1024 * 1024, seed=1, chunk=1 << 21):
        import torch

        xs, ys, gs, ws = [], [], [], []
        for i, s in enumerate(range(0, n_samples, chunk)):
            m = min(chunk, n_samples - s)
            x = self.sample_positions(m, seed * 1000 + i)
            xh, ystar, gstar, wg = self.targets(x)
            xs.append(xh.T.float())
            ys.append(ystar.float())
            gs.append(gstar.T.float())
            ws.append(wg)
        self.X = torch.cat(xs).contiguous()
        self.Y = torch.cat(ys).contiguous()
        self.Gt = torch.cat(gs).contiguous()
        w = torch.cat(ws)
        self.Wg = (w / w.mean()).float().contiguous()
        self.y_scale = float(self.Y.std())
        return self.X.shape[0]

    # ------------------------------------------------------------ training
    @traced("surrogate_train")
    def train(self, steps=6000, batch=8192, lr=1e-3, lr_min=1e-5, beta=4.0, seed=2, log_every=500,
              qat_fraction=0.3):
        """Adam with cosine learning-rate decay on minibatches of the dataset.
        The targets are divided by y_scale during training; the scale is folded
        into the output layer afterwards.  For the last `qat_fraction` of the
        steps the 256 x 256 weights are rounded to BF16 for the forward and
        backward passes (the update goes to the FP32 weights)."""
        import torch

        from ._device import ptr, stream_handle

        s = self.y_scale
        Ys, Gs = self.Y / s, self.Gt / s
        m = torch.zeros_like(self.params)
        v = torch.zeros_like(self.params)
        grads = torch.zeros_like(self.params)
        ws = torch.empty(int(_abi.load().gx_mlp_train_workspace_floats(batch)), dtype=torch.float32, device=self.dev)
        loss = torch.zeros(2, dtype=torch.float32, device=self.dev)
        gen = torch.Generator(device=self.dev)
        gen.manual_seed(seed)
        N = self.X.shape[0]
        lib = _abi.load()
        h = stream_handle()
        qp = self.params.clone()
        qat_start = int(steps * (1.0 - qat_fraction)) + 1
        qdt = torch.float16 if self.split == 3 else torch.bfloat16   # the inference operand type
        big = [(o, o + H * H) for o in (OFF_W2, OFF_W3, OFF_W4)]
        for step in range(1, steps + 1):
            idx = torch.randint(0, N, (batch,), generator=gen, device=self.dev)
            xb, yb, gb = self.X[idx].contiguous(), Ys[idx].contiguous(), Gs[idx].contiguous()
            wb = self.Wg[idx].contiguous()
            use = self.params
            if step >= qat_start:
                qp.copy_(self.params)
                for a, b in big:
                    qp[a:b] = self.params[a:b].to(qdt).float()
                use = qp
            _abi.call("gx_mlp_train_step", ptr(use), ptr(grads), ptr(xb), ptr(yb), ptr(gb), ptr(wb), batch,
                      C.c_float(1.0), C.c_float(beta), ptr(ws), ptr(loss), h)
            lr_t = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * step / steps))
            _abi.call("gx_mlp_adam", ptr(self.params), ptr(grads), ptr(m), ptr(v), NPARAM, C.c_float(lr_t),
                      C.c_float(0.9), C.c_float(0.999), C.c_float(1e-8), step, h)
            if step % log_every == 0 or step == steps:
                lv, lg = loss.tolist()
                self.history.append((step, lv, lg))
        del lib
        # fold the target scale into the output layer
        self.params[OFF_W5:OFF_B5] *= s
        self.params[OFF_B5] *= s
        self.export()
        return self.history

    def export(self):
        """BF16 weight pack for inference: W2, W3, W4, W4^T, W3^T, W2^T, and its
        tensor-core image (64-wide K chunks, 128-byte swizzle; see
        gx_surrogate_gradient_tc in include/gala_gb300.h)."""
        import torch

        Ws = [self.params[o:o + H * H].view(H, H) for o in (OFF_W2, OFF_W3, OFF_W4)]
        pack = [Ws[0], Ws[1], Ws[2], Ws[2].T, Ws[1].T, Ws[0].T]
        self.wbf16 = torch.stack([w.contiguous() for w in pack]).to(torch.bfloat16).contiguous()
        # [matrix][row][chunk][granule][8] -> [matrix][chunk][row][granule ^ (row & 7)][8]
        self.wimg = self._image(self.wbf16)
        self.wimg16 = self._image(torch.stack([w.contiguous() for w in pack]).to(torch.float16).contiguous())
        return self.wbf16

    @staticmethod
    def _image(w16):
        """Tensor-core image of six 256 x 256 16-bit matrices (BF16 or FP16):
        64-wide K chunks with the 128-byte swizzle."""
        import torch

        v = w16.view(6, H, H // 64, 8, 8).permute(0, 2, 1, 3, 4).contiguous()
        rows = torch.arange(H, device=v.device)
        src = (torch.arange(8, device=v.device)[None, :] ^ (rows[:, None] & 7))  # [row][dest granule] -> source
        idx = src.view(1, 1, H, 8, 1).expand(6, H // 64, H, 8, 8)
        return torch.gather(v, 3, idx).contiguous()

    def _tc_image(self):
        return self.wimg16 if self.split == 3 else self.wimg

    # ------------------------------------------------------------ inference
    def _grid(self, n, tile=64):
        import torch

        sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        return int(max(1, min(sms, (n + tile - 1) // tile)))

    @traced("surrogate_gradient")
    def gradient_and_energy(self, q, engine=None):
        """grad Phi (3, N) and Phi (N) at positions q (3, N), on the tensor cores:
        engine "tcgen05" (default) or "mma" (warp-level mma.sync)."""
        engine = engine or self.engine
        import torch

        from ._device import as_device_f64, ptr, stream_handle

        if self.wbf16 is None:
            self.export()
        qd = as_device_f64(q).reshape(3, -1).contiguous()
        n = qd.shape[1]
        grad = torch.empty((3, n), dtype=torch.float64, device=self.dev)
        phi = torch.empty(n, dtype=torch.float64, device=self.dev)
        if engine == "tcgen05":
            status = torch.zeros(1, dtype=torch.int32, device=self.dev)
            _abi.call("gx_surrogate_gradient_tc", ptr(self.params), ptr(self._tc_image()), ptr(self.scf_f32), self.r_min,
                      self.r_max, self.GM, self.r_s, self.split, ptr(qd), n, ptr(grad), ptr(phi),
                      self._grid(n, 128), ptr(status), stream_handle())
            self._check(status)
        else:
            # the warp-level engine has BF16 operands only (split 1 or 2)
            _abi.call("gx_surrogate_gradient", ptr(self.params), ptr(self.wbf16), ptr(self.scf_f32), self.r_min,
                      self.r_max, self.GM, self.r_s, min(self.split, 2), ptr(qd), n, ptr(grad), ptr(phi), self._grid(n),
                      stream_handle())
        return grad, phi

    @staticmethod
    def _check(status):
        if int(status.item()) != 0:
            raise _abi.GxError("the tensor-core surrogate kernel ran out of a bounded wait (results incomplete)")

    @traced("surrogate_leapfrog")
    def integrate_leapfrog(self, w0, dt, n_steps, grid=None, analytic=False, engine=None):
        """FP32 leapfrog of every orbit in w0 (6, N) in the surrogate potential;
        returns the final states (6, N) and the number of fallback force calls.
        analytic=True: the same integrator with the analytic SCF force (FP32)
        for every evaluation, i.e. without the surrogate."""
        import torch

        from ._device import as_device_f64, ptr, stream_handle

        if self.wbf16 is None and not analytic:
            self.export()
        w0d = as_device_f64(w0)
        n = w0d.shape[1]
        out = torch.empty_like(w0d)
        fb = torch.zeros(1, dtype=torch.int64, device=self.dev)
        if (engine or self.engine) == "tcgen05" and not analytic:
            status = torch.zeros(1, dtype=torch.int32, device=self.dev)
            _abi.call("gx_surrogate_leapfrog_tc", ptr(self.params), ptr(self._tc_image()), ptr(self.scf_f32), self.r_min,
                      self.r_max, self.GM, self.r_s, self.split, ptr(w0d), n, int(n_steps), float(dt), ptr(out),
                      ptr(fb), grid or self._grid(n, 128), ptr(status), stream_handle())
            self._check(status)
            return out, fb
        wb = ptr(self.wbf16) if self.wbf16 is not None else None
        _abi.call("gx_surrogate_leapfrog", ptr(self.params), wb, ptr(self.scf_f32), self.r_min,
                  self.r_max, self.GM, self.r_s, min(self.split, 2), int(bool(analytic)), ptr(w0d), n, int(n_steps),
                  float(dt), ptr(out), ptr(fb), grid or self._grid(n), stream_handle())
        return out, fb

    # ------------------------------------------------------------ files
    def save(self, path):
        """Write the trained network (FP32 weights with the target scale folded
        in) and its input box to an .npz file."""
        np.savez(path, params=self.params.cpu().numpy(), r_min=self.r_min, r_max=self.r_max, split=self.split,
                 scf_params=self.scf.packed().params)

    @classmethod
    def load(cls, path, scf):
        """A network written by save(), for the same SCF potential `scf` (its
        packed parameters must match the file's)."""
        import torch

        d = np.load(path)
        if not np.array_equal(d["scf_params"], scf.packed().params):
            raise ValueError(f"{path} was trained for a different SCF potential")
        sp = cls(scf, r_min=float(d["r_min"]), r_max=float(d["r_max"]), split=int(d["split"]))
        sp.params = torch.from_numpy(np.ascontiguousarray(d["params"], dtype=np.float32)).to(sp.dev)
        sp.export()
        return sp

    def forward_fp32(self, xh):
        """Network value and input gradient in FP32 (training kernels), xh (N, 3)."""
        import torch

        from ._device import ptr, stream_handle

        xh = xh.to(self.dev, torch.float32).contiguous()
        B = xh.shape[0]
        y = torch.empty(B, dtype=torch.float32, device=self.dev)
        G = torch.empty((B, 3), dtype=torch.float32, device=self.dev)
        ws = torch.empty(int(_abi.load().gx_mlp_train_workspace_floats(B)), dtype=torch.float32, device=self.dev)
        _abi.call("gx_mlp_forward", ptr(self.params), ptr(xh), B, ptr(y), ptr(G), ptr(ws), stream_handle())
        return y, G

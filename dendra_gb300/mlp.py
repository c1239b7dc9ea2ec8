"""BF16 tensor-core MLP that proposes activation-threshold brackets.

Maps fibre and stimulus parameters (log D, log distance, axial offset,
log pulse width; standardised) to the log threshold (standardised).  Layers
4 -> 256 -> 256 -> 256 -> 1 with exact GELU between them; BF16 weights and
activations, FP32 accumulation, FP32 master weights trained with Adam.
Every forward, backward and optimizer operation runs in the library's
kernels (``dgb_mlp_gemm``, ``dgb_colsum``, ``dgb_adam``, ``dgb_mse_grad``);
the 256-wide hidden-layer products (forward and dH) run on tcgen05 tensor
cores fed by TMA whenever the batch is a multiple of 128 rows.

The reference has no learned component: the proposal only narrows the
bracket that the plain bisection (threshold.Thresholder) then confirms.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib

EPI_PLAIN, EPI_BIAS, EPI_BIAS_GELU, EPI_GELU_GRAD = 0, 1, 2, 3

MLP_FLOPS_NOTE = ("inference FLOPs 2*(4*256 + 2*256*256 + 256) per sample over the forward "
                  "time (4 launches): the two 256x256 layers on tcgen05 (128x256 tiles, TMA "
                  "128-byte swizzle, TMEM accumulator), the K = 4 input and N = 1 output "
                  "layers on mma.sync")


def _gemm(M, N, K, A, sam, sak, B, sbk, sbn, *, bias=None, epi=EPI_PLAIN, aux=None, out32=None,
          out16=None):
    dev = A.device
    with torch.cuda.device(dev):
        rc = _lib.load().dgb_mlp_gemm(
            M, N, K, A.data_ptr(), sam, sak, B.data_ptr(), sbk, sbn,
            None if bias is None else bias.data_ptr(), epi,
            None if aux is None else aux.data_ptr(),
            None if out32 is None else out32.data_ptr(),
            None if out16 is None else out16.data_ptr(), _lib.stream_ptr(dev))
    _lib.check(rc, "dgb_mlp_gemm")


def gemm_status(device) -> None:
    """Raise ``DgbTimeout`` if a bounded wait inside the last tcgen05 GEMM on
    ``device`` gave up (that GEMM's output is then invalid).  Synchronises the
    current stream."""
    with torch.cuda.device(device):
        rc = _lib.load().dgb_mlp_gemm_status(_lib.stream_ptr(device))
    _lib.check(rc, "tcgen05 GEMM")


class BF16MLP:
    def __init__(self, dims=(4, 256, 256, 256, 1), device="cuda", seed=0):
        self.dims = tuple(dims)
        self.device = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        self.W, self.b = [], []
        for k, n in zip(self.dims[:-1], self.dims[1:]):
            bound = 1.0 / np.sqrt(k)
            self.W.append(((torch.rand(k, n, generator=g) * 2 - 1) * bound).to(self.device))
            self.b.append(((torch.rand(n, generator=g) * 2 - 1) * bound).to(self.device))
        self.W16 = [w.to(torch.bfloat16) for w in self.W]
        # K-major copies [N][K]: the forward's B operand for the tcgen05 path
        self.Wt16 = [w.t().contiguous().to(torch.bfloat16) for w in self.W]
        self.opt = None
        self.x_mean = self.x_std = None
        self.y_mean, self.y_std = 0.0, 1.0

    # -- forward / backward on the kernels --------------------------------
    def forward(self, x16, keep=False):
        """x16: (M, d_in) bf16.  Returns y (M, d_out) fp32 (and activations when keep)."""
        M = x16.shape[0]
        h = x16
        acts = [h]
        zs = []
        L = len(self.W)
        for li, (Wt16, b) in enumerate(zip(self.Wt16, self.b)):
            N, K = Wt16.shape
            z = torch.empty(M, N, dtype=torch.float32, device=self.device)
            # B[k, n] = W[k, n] read K-major from W^T (sbk = 1, sbn = K)
            if li < L - 1:
                hn = torch.empty(M, N, dtype=torch.bfloat16, device=self.device)
                _gemm(M, N, K, h, K, 1, Wt16, 1, K, bias=b, epi=EPI_BIAS_GELU, out32=z, out16=hn)
                h = hn
                acts.append(h)
            else:
                _gemm(M, N, K, h, K, 1, Wt16, 1, K, bias=b, epi=EPI_BIAS, out32=z)
            zs.append(z)
        return (zs[-1], acts, zs) if keep else zs[-1]

    def backward(self, dy16, acts, zs):
        """Gradients (dW list, db list) for the output gradient dy16 (M, d_out) bf16."""
        M = dy16.shape[0]
        L = len(self.W)
        dW = [None] * L
        db = [None] * L
        dz16 = dy16
        dz32 = None
        for li in range(L - 1, -1, -1):
            K, N = self.W16[li].shape
            h = acts[li]
            gw = torch.empty(K, N, dtype=torch.float32, device=self.device)
            # dW[k, n] = sum_m h[m, k] dz[m, n]
            _gemm(K, N, M, h, 1, K, dz16, N, 1, epi=EPI_PLAIN, out32=gw)
            dW[li] = gw
            gb = torch.empty(N, dtype=torch.float32, device=self.device)
            if dz32 is None:
                dz32 = dz16.float()
            with torch.cuda.device(self.device):
                rc = _lib.load().dgb_colsum(M, N, dz32.data_ptr(), gb.data_ptr(),
                                            _lib.stream_ptr(self.device))
            _lib.check(rc, "dgb_colsum")
            db[li] = gb
            if li > 0:
                # dh[m, k] = sum_n dz[m, n] W[k, n]; dz_prev = dh * gelu'(z_prev)
                nz16 = torch.empty(M, K, dtype=torch.bfloat16, device=self.device)
                nz32 = torch.empty(M, K, dtype=torch.float32, device=self.device)
                _gemm(M, K, N, dz16, N, 1, self.W16[li], 1, N, epi=EPI_GELU_GRAD,
                      aux=zs[li - 1], out32=nz32, out16=nz16)
                dz16, dz32 = nz16, nz32
        return dW, db

    # -- training ---------------------------------------------------------
    def _adam(self, params, grads, lr, step):
        if self.opt is None:
            self.opt = [(torch.zeros_like(p), torch.zeros_like(p)) for p in params]
        L = _lib.load()
        for i, (p, g) in enumerate(zip(params, grads)):
            m1, m2 = self.opt[i]
            w16 = self.W16[i // 2] if i % 2 == 0 else None
            wt16 = self.Wt16[i // 2] if i % 2 == 0 else None
            K, N = (p.shape if p.ndim == 2 else (1, p.numel()))
            with torch.cuda.device(self.device):
                rc = L.dgb_adam(p.numel(), N, K, p.data_ptr(), g.data_ptr(), m1.data_ptr(),
                                m2.data_ptr(), lr, 0.9, 0.999, 1e-8, step,
                                None if w16 is None else w16.data_ptr(),
                                None if wt16 is None else wt16.data_ptr(),
                                _lib.stream_ptr(self.device))
            _lib.check(rc, "dgb_adam")

    def standardize_fit(self, X, y):
        self.x_mean = X.mean(0).to(self.device)
        self.x_std = X.std(0).clamp_min(1e-6).to(self.device)
        self.y_mean = float(y.mean())
        self.y_std = float(y.std().clamp_min(1e-6))

    def _inputs(self, X):
        return ((X - self.x_mean) / self.x_std).to(torch.bfloat16).contiguous()

    def train(self, X, y, epochs=30, batch=4096, lr=2e-3, seed=0):
        """X (M, 4) fp32 features, y (M,) fp32 targets (log threshold)."""
        if self.x_mean is None:
            self.standardize_fit(X, y)
        Xs = self._inputs(X.to(self.device))
        ys = ((y.to(self.device) - self.y_mean) / self.y_std).float().reshape(-1, 1).contiguous()
        M = Xs.shape[0]
        g = torch.Generator(device="cpu").manual_seed(seed)
        step = 0
        L = _lib.load()
        losses = []
        for ep in range(epochs):
            perm = torch.randperm(M, generator=g).to(self.device)
            for s0 in range(0, M - batch + 1, batch):
                idx = perm[s0:s0 + batch]
                xb, yb = Xs[idx].contiguous(), ys[idx].contiguous()
                out, acts, zs = self.forward(xb, keep=True)
                dy16 = torch.empty_like(out, dtype=torch.bfloat16)
                with torch.cuda.device(self.device):
                    rc = L.dgb_mse_grad(out.numel(), out.data_ptr(), yb.data_ptr(),
                                        2.0 / out.numel(), None, dy16.data_ptr(),
                                        _lib.stream_ptr(self.device))
                _lib.check(rc, "dgb_mse_grad")
                dW, db = self.backward(dy16, acts, zs)
                step += 1
                lr_t = lr * min(1.0, 0.5 * (1 + np.cos(np.pi * step / (epochs * (M // batch)))) + 0.02)
                params = [p for pair in zip(self.W, self.b) for p in pair]
                grads = [q for pair in zip(dW, db) for q in pair]
                self._adam(params, grads, lr_t, step)
            gemm_status(self.device)
            losses.append(float(((out - yb) ** 2).mean()))
        return losses

    def predict(self, X):
        """Predicted targets (de-standardised) for features X (M, 4)."""
        out = self.forward(self._inputs(X.to(self.device)))
        gemm_status(self.device)
        return out.reshape(-1) * self.y_std + self.y_mean


def fibre_features(p):
    """(log D, log distance, axial offset, log pulse width) as an (M, 4) tensor."""
    return torch.as_tensor(np.stack([np.log(p["D"]), np.log(p["dist"]), p["offset"],
                                     np.log(p["pw"])], axis=1), dtype=torch.float32)

"""Learned band for global alignment: features, training and inference of the band predictor.

The predictor is a BF16 MLP 130 -> 256 -> 256 -> 9 whose kernels are this
project's own (``pa_mlp_*`` in csrc/pa_band.cu: a tensor-core BF16 GEMM with FP32
accumulation and a fused bias/ReLU epilogue, the MSE gradient, the ReLU
derivative, bias gradients and Adam).  torch only allocates device memory.

Inputs (``features``): the 128-bin histogram of diagonal offsets of shared
12-mers plus both lengths (``pa_band_features_device``).
Targets (``targets``): the 8 optimal-path diagonals at the checkpoint columns
i_c = (c+1)*m/9 of sequence1, from the full GPU DP (``pa_band_labels``), scaled
by 4/(m+n), and log2(1 + c2)/16 where c2 = smax*(m+n) - 2*score is the score
deficit of the optimal alignment.  The library decodes the outputs on the
device (k_band_decode): the centre line runs through (0, 0), the predicted
checkpoints and (m, n); a path that leaves the band must pay the deficit in
gaps, which sets the starting half-width.  The band is only a proposal: the
banded DP proves its score with an admissible bound, doubles the band when it
cannot, and falls back to the full DP.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib

FEAT, FEAT_PAD, HIDDEN, OUT, OUT_PAD = 130, 144, 256, 9, 16


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _check(rc):
    _lib.check(rc)


def features(seq1_dev, off1_dev, seq2_dev, off2_dev, stream=None):
    """Device tensors in -> (n_pairs, 130) float32 device tensor of band features."""
    import torch
    n = off1_dev.numel() - 1
    out = torch.empty((max(n, 1), FEAT), dtype=torch.float32, device=seq1_dev.device)
    h = getattr(stream, "cuda_stream", None) if stream is not None else None
    _check(_lib.load().pa_band_features_device(_p(seq1_dev), _p(off1_dev), _p(seq2_dev), _p(off2_dev), n, _p(out),
                                               h))
    return out[:n]


def labels(context, c_config, seq1, off1, seq2, off2) -> np.ndarray:
    """Host arrays in -> (n_pairs, 8) int32 optimal-path diagonals at the checkpoints (full GPU DP)."""
    n = len(off1) - 1
    seq1 = np.ascontiguousarray(seq1, dtype=np.uint8)
    seq2 = np.ascontiguousarray(seq2, dtype=np.uint8)
    off1 = np.ascontiguousarray(off1, dtype=np.uint64)
    off2 = np.ascontiguousarray(off2, dtype=np.uint64)
    out = np.zeros((max(n, 1), 8), dtype=np.int32)
    _lib.check(context.lib.pa_band_labels(context.ptr, ctypes.byref(c_config), seq1.ctypes.data, off1.ctypes.data,
                                          seq2.ctypes.data, off2.ctypes.data, n, out.ctypes.data), context.ptr)
    return out[:n]


def targets(lab: np.ndarray, m: np.ndarray, n: np.ndarray, score: np.ndarray, smax: int) -> np.ndarray:
    """(n_pairs, 9) float32 training targets: the checkpoint diagonals scaled by 4 / (m + n), and
    log2(1 + c2) / 16 with c2 = smax (m + n) - 2 score, the score deficit the band width is sized by."""
    lab = lab.astype(np.float64)
    mn = (m + n).astype(np.float64)
    y = np.zeros((len(lab), OUT), dtype=np.float32)
    y[:, :8] = lab * (4.0 / np.maximum(mn, 1.0))[:, None]
    c2 = np.maximum(smax * mn - 2.0 * score.astype(np.float64), 0.0)
    y[:, 8] = np.log2(1.0 + c2) / 16.0
    return y


def band_centres(pred: np.ndarray, m: np.ndarray, n: np.ndarray):
    """Predicted checkpoint diagonals (n_pairs, 8) and score deficits c2 (n_pairs,) from network outputs."""
    d = np.rint(pred[:, :8].astype(np.float64) * (m + n)[:, None] / 4.0).astype(np.int64)
    c2 = 2.0 ** (16.0 * np.minimum(pred[:, 8].astype(np.float64), 1.5)) - 1.0
    return d, c2


class BandModel:
    """Parameters and buffers of the band predictor on one device."""

    def __init__(self, device="cuda:0", seed: int = 0, max_batch: int = 4096):
        import torch
        self.torch = torch
        self.dev = torch.device(device)
        g = np.random.default_rng(seed)

        def init(fan_in, shape):
            return torch.from_numpy((g.standard_normal(shape) * math.sqrt(2.0 / fan_in)).astype(np.float32))

        shapes = {"W1": (FEAT_PAD, HIDDEN), "b1": (HIDDEN,), "W2": (HIDDEN, HIDDEN), "b2": (HIDDEN,),
                  "W3": (HIDDEN, OUT_PAD), "b3": (OUT_PAD,)}
        self.w = {}
        for k, shp in shapes.items():
            if k.startswith("W"):
                t = init(shp[0], shp)
                if k == "W1":
                    t[FEAT:, :] = 0.0
                if k == "W3":
                    t[:, OUT:] = 0.0
            else:
                t = torch.zeros(shp)
            self.w[k] = t.to(self.dev)
        self.w16 = {k: v.to(torch.bfloat16) for k, v in self.w.items() if k.startswith("W")}
        self.m1 = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.m2 = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.g = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.step_no = 0
        self._alloc(max_batch)

    def _alloc(self, B):
        t = self.torch
        self.B = B
        self.x16 = t.zeros((B, FEAT_PAD), dtype=t.bfloat16, device=self.dev)
        self.h1 = t.zeros((B, HIDDEN), dtype=t.bfloat16, device=self.dev)
        self.h2 = t.zeros((B, HIDDEN), dtype=t.bfloat16, device=self.dev)
        self.out = t.zeros((B, OUT_PAD), dtype=t.float32, device=self.dev)
        self.dout = t.zeros((B, OUT_PAD), dtype=t.bfloat16, device=self.dev)
        self.dh2 = t.zeros((B, HIDDEN), dtype=t.bfloat16, device=self.dev)
        self.dh1 = t.zeros((B, HIDDEN), dtype=t.bfloat16, device=self.dev)
        self.loss = t.zeros(1, dtype=t.float32, device=self.dev)

    # -- kernels ---------------------------------------------------------------
    def _gemm(self, A, Bm, C32, C16, bias, M, N, K, lda, ldb, ldc, ta, tb, relu, beta=0.0):
        _check(_lib.load().pa_mlp_gemm(_p(A), _p(Bm), _p(C32), _p(C16), _p(bias), M, N, K, lda, ldb, ldc, ta, tb,
                                       relu, beta, None))

    def forward(self, x32, B: int):
        """x32: (B, 130) float32 device tensor -> out (B, 16) float32 (first 9 used)."""
        L = _lib.load()
        if B > self.B:
            self._alloc(B)
        _check(L.pa_mlp_to_bf16(_p(x32), B, FEAT, FEAT_PAD, _p(self.x16), None))
        self._gemm(self.x16, self.w16["W1"], None, self.h1, self.w["b1"], B, HIDDEN, FEAT_PAD, FEAT_PAD, HIDDEN,
                   HIDDEN, 0, 0, 1)
        self._gemm(self.h1, self.w16["W2"], None, self.h2, self.w["b2"], B, HIDDEN, HIDDEN, HIDDEN, HIDDEN, HIDDEN,
                   0, 0, 1)
        self._gemm(self.h2, self.w16["W3"], self.out, None, self.w["b3"], B, OUT_PAD, HIDDEN, HIDDEN, OUT_PAD,
                   OUT_PAD, 0, 0, 0)
        return self.out[:B]

    def backward(self, y32, mask32, B: int) -> None:
        """Gradients of the mean squared error into self.g (after forward on the same batch)."""
        L = _lib.load()
        self.loss.zero_()
        _check(L.pa_mlp_mse(_p(self.out), _p(y32), _p(mask32), B, _p(self.dout), _p(self.loss), None))
        # layer 3
        self._gemm(self.h2, self.dout, self.g["W3"], None, None, HIDDEN, OUT_PAD, B, HIDDEN, OUT_PAD, OUT_PAD, 1, 0, 0)
        _check(L.pa_mlp_colsum(_p(self.dout), B, OUT_PAD, _p(self.g["b3"]), None))
        self._gemm(self.dout, self.w16["W3"], None, self.dh2, None, B, HIDDEN, OUT_PAD, OUT_PAD, OUT_PAD, HIDDEN,
                   0, 1, 0)
        _check(L.pa_mlp_relu_grad(_p(self.dh2), _p(self.h2), B * HIDDEN, None))
        # layer 2
        self._gemm(self.h1, self.dh2, self.g["W2"], None, None, HIDDEN, HIDDEN, B, HIDDEN, HIDDEN, HIDDEN, 1, 0, 0)
        _check(L.pa_mlp_colsum(_p(self.dh2), B, HIDDEN, _p(self.g["b2"]), None))
        self._gemm(self.dh2, self.w16["W2"], None, self.dh1, None, B, HIDDEN, HIDDEN, HIDDEN, HIDDEN, HIDDEN, 0, 1, 0)
        _check(L.pa_mlp_relu_grad(_p(self.dh1), _p(self.h1), B * HIDDEN, None))
        # layer 1
        self._gemm(self.x16, self.dh1, self.g["W1"], None, None, FEAT_PAD, HIDDEN, B, FEAT_PAD, HIDDEN, HIDDEN, 1,
                   0, 0)
        _check(L.pa_mlp_colsum(_p(self.dh1), B, HIDDEN, _p(self.g["b1"]), None))

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, weight_decay=0.0):
        L = _lib.load()
        self.step_no += 1
        for k in self.w:
            w16 = self.w16.get(k)
            _check(L.pa_mlp_adam(_p(self.w[k]), _p(w16), _p(self.g[k]), _p(self.m1[k]), _p(self.m2[k]),
                                 self.w[k].numel(), lr, b1, b2, eps, self.step_no, weight_decay, None))
        # the padding rows / columns of W1 and W3 stay zero
        self.w["W1"][FEAT:, :] = 0.0
        self.w16["W1"][FEAT:, :] = 0.0
        self.w["W3"][:, OUT:] = 0.0
        self.w16["W3"][:, OUT:] = 0.0
        self.w["b3"][OUT:] = 0.0

    def train(self, x: "np.ndarray", y: "np.ndarray", mask: "np.ndarray", epochs: int = 3, batch: int = 4096,
              lr: float = 1e-3, seed: int = 0, log=None) -> list[float]:
        t = self.torch
        n = len(x)
        xd = t.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(self.dev)
        yd = t.from_numpy(np.ascontiguousarray(y, dtype=np.float32)).to(self.dev)
        md = t.from_numpy(np.ascontiguousarray(mask, dtype=np.float32)).to(self.dev)
        rng = np.random.default_rng(seed)
        hist = []
        for ep in range(epochs):
            perm = t.from_numpy(rng.permutation(n)).to(self.dev)
            tot, cnt = 0.0, 0
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                xb, yb, mb = xd[idx].contiguous(), yd[idx].contiguous(), md[idx].contiguous()
                self.forward(xb, batch)
                self.backward(yb, mb, batch)
                self.adam(lr=lr)
                tot += float(self.loss.item()) / (batch * OUT)
                cnt += 1
            hist.append(tot / max(cnt, 1))
            if log:
                log(f"epoch {ep}: mse {hist[-1]:.5f}")
        return hist

    def predict(self, x32_dev) -> np.ndarray:
        n = x32_dev.shape[0]
        out = np.zeros((n, OUT), dtype=np.float32)
        for s in range(0, n, self.B):
            b = min(self.B, n - s)
            bp = ((b + 63) // 64) * 64
            xb = self.torch.zeros((bp, FEAT), dtype=self.torch.float32, device=self.dev)
            xb[:b] = x32_dev[s:s + b]
            o = self.forward(xb, bp)
            out[s:s + b] = o[:b, :OUT].cpu().numpy()
        return out

    def state(self) -> dict:
        return {k: v.detach().cpu().numpy() for k, v in self.w.items()}

    def load_state(self, st: dict):
        t = self.torch
        for k, v in st.items():
            self.w[k] = t.from_numpy(np.asarray(v, dtype=np.float32)).to(self.dev)
            if k.startswith("W"):
                self.w16[k] = self.w[k].to(t.bfloat16)

    def to_context(self, context) -> None:
        """Load the current weights into a Context for band_mode 1."""
        context.set_band_model(self.state())

    def save(self, path: str):
        np.savez(path, step=self.step_no, **self.state())

    def load(self, path: str):
        z = np.load(path)
        self.load_state({k: z[k] for k in z.files if k != "step"})
        self.step_no = int(z["step"])

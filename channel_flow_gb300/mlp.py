"""Learned initial guess of the pseudo-time iterations.

A per-cell MLP maps the 3x3x3 neighbourhood of the last two time
increments dU^n = U^n - U^(n-1) and dU^(n-1) = U^(n-1) - U^(n-2) of the
five conserved variables, presented as dU^n and d2U = dU^n - dU^(n-1)
(2 x 27 x 5 = 270 features, each kind scaled per variable by its interior
RMS; the second difference is formed in FP64, because in BF16 the two
increments agree to about the digits that their difference needs), through
two hidden layers of 128 SiLU units to the five components of the error of
a linear predictor P = U^n + a_v dU^n + b_v d2U of U^(n+1) (in units of the
RMS second difference times a per-variable factor fitted on the training
windows).  a_v and b_v are least-squares fits over the training windows:
a smooth transient gives about the quadratic extrapolation (a = b = 1), an
oscillating one (acoustic waves of the initial state) about the plain
start U^n (a = b = 0), which the quadratic extrapolation then overshoots.
The network corrects the predictor rather than predicting the increment
itself, so its BF16 precision limits only the small correction, and a
least-squares gain per variable, fitted on a held-out window, scales a
correction that does not help there towards zero.  Before the
sub-iterations of a physical step the state starts from that guess instead
of U^n; the sub-iterations still run to the same residual tolerance, so the
plain LU-SGS loop still decides convergence and remains the fallback.

Every matrix product runs on the tcgen05 tensor cores (``cf_gemm_bf16``,
BF16 operands, FP32 accumulation) and every other step in the package's own
kernels (``cf_mlp_*``); PyTorch only holds the device buffers.  Training is
Adam on the mean squared error over windows harvested from the solver's own
steps.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

IN, K1, H, OUT, N3, K3 = 270, 320, 128, 5, 16, 64
EPI_F32, EPI_SILU, EPI_BIAS = 0, 1, 2
WGRAD_PARTIAL = 1 << 23          # floats of split-K partial products (32 MB)

# flat parameter vector: W1 [128 x 320], b1 [128], W2 [128 x 128], b2 [128],
# W3T [128 x 16] (the transposed output layer), b3 [16]
_SHAPES = [("W1", (H, K1)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3T", (H, N3)), ("b3", (N3,))]


def _offsets():
    off, out = 0, {}
    for n, s in _SHAPES:
        size = int(np.prod(s))
        out[n] = (off, s)
        off += size
    return out, off


OFFS, NPARAM = _offsets()


def init_params(seed: int = 0) -> np.ndarray:
    """Seeded initial parameters (scaled normal weights, zero biases; the
    padded feature columns and output rows are zero)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, np.float32)

    def put(name, val):
        o, s = OFFS[name]
        p[o:o + int(np.prod(s))] = val.astype(np.float32).ravel()
    W1 = np.zeros((H, K1))
    W1[:, :IN] = rng.normal(0, np.sqrt(1.0 / IN), (H, IN))
    put("W1", W1)
    put("W2", rng.normal(0, np.sqrt(1.0 / H), (H, H)))
    W3T = np.zeros((H, N3))
    W3T[:, :OUT] = rng.normal(0, 0.1 * np.sqrt(1.0 / H), (H, OUT))
    put("W3T", W3T)
    return p


def _pad(m: int) -> int:
    return (m + 255) // 256 * 256


class LearnedGuess:
    """The MLP on one device; ``capacity`` rows per forward/training call."""

    def __init__(self, capacity: int = 32768, seed: int = 0, lr: float = 1e-3, batch: int | None = None):
        """``capacity``: rows of one inference pass (the grid's cells for
        ``guess``); ``batch``: rows of one training step (default capacity)."""
        import torch
        self.torch = torch
        self.lib = _lib.load()
        self.cap = _pad(capacity)
        self.tcap = self.cap if batch is None else min(_pad(batch), self.cap)
        dev = "cuda"
        f32, bf = torch.float32, torch.bfloat16
        self.p = torch.from_numpy(init_params(seed)).to(dev)
        self.g = torch.zeros(NPARAM, dtype=f32, device=dev)
        self.m = torch.zeros(NPARAM, dtype=f32, device=dev)
        self.v = torch.zeros(NPARAM, dtype=f32, device=dev)
        self.t = 0
        self.lr = lr
        self.W1b = torch.zeros(H, K1, dtype=bf, device=dev)
        self.W2b = torch.zeros(H, H, dtype=bf, device=dev)
        self.W3b = torch.zeros(N3, H, dtype=bf, device=dev)
        self.W2T = torch.zeros(H, H, dtype=bf, device=dev)
        self.W3p = torch.zeros(H, K3, dtype=bf, device=dev)
        # inference-sized buffers
        M = self.cap
        self.X = torch.zeros(M, K1, dtype=bf, device=dev)
        self.H1 = torch.zeros(M, H, dtype=bf, device=dev)
        self.H2 = torch.zeros(M, H, dtype=bf, device=dev)
        self.Y = torch.zeros(M, N3, dtype=f32, device=dev)
        # training-sized buffers
        M = self.tcap
        self.Z1 = torch.zeros(M, H, dtype=f32, device=dev)
        self.Z2 = torch.zeros(M, H, dtype=f32, device=dev)
        self.T = torch.zeros(M, N3, dtype=f32, device=dev)
        self.dY = torch.zeros(M, K3, dtype=bf, device=dev)
        self.dYT = torch.zeros(N3, M, dtype=bf, device=dev)
        self.dH = torch.zeros(M, H, dtype=f32, device=dev)
        self.dZ2 = torch.zeros(M, H, dtype=bf, device=dev)
        self.dZ2T = torch.zeros(H, M, dtype=bf, device=dev)
        self.dZ1 = torch.zeros(M, H, dtype=bf, device=dev)
        self.dZ1T = torch.zeros(H, M, dtype=bf, device=dev)
        self.H1T = torch.zeros(H, M, dtype=bf, device=dev)
        self.H2T = torch.zeros(H, M, dtype=bf, device=dev)
        self.XT = torch.zeros(K1, M, dtype=bf, device=dev)
        self.partial = torch.zeros(M // 256 * 6, dtype=f32, device=dev)
        self.rms_partial = torch.zeros(30 * 512, dtype=torch.float64, device=dev)
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        # split-K partial products of the weight gradients (their outputs are
        # one to five 128-row tiles, their reduction runs over the rows)
        self.sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        self.wpart = torch.zeros(WGRAD_PARTIAL, dtype=f32, device=dev)
        self.scale = torch.ones(10, dtype=f32, device=dev)
        self.coef = np.ones(10)                             # predictor a[0..4], b[5..9] (quadratic extrapolation)
        self.D = None                                       # FP32 time differences of the whole-grid feature rows
        self.oscale = torch.ones(5, dtype=f32, device=dev)   # output unit of the network (targets)
        self.ogain = torch.ones(5, dtype=f32, device=dev)    # oscale times the fitted gain (the guess)
        self.gen = torch.Generator(device=dev)
        self.gen.manual_seed(seed + 7919)
        self.validation = None
        self.updates = []
        self.pack()

    # -- helpers ----------------------------------------------------------
    def _s(self):
        return self.torch.cuda.current_stream().cuda_stream

    def _ok(self, rc, what):
        if rc != _lib.CF_OK:
            raise RuntimeError(f"{what} failed with status {rc}")

    def view(self, name, t=None):
        o, s = OFFS[name]
        t = self.p if t is None else t
        return t[o:o + int(np.prod(s))].view(*s)

    def pack(self):
        """fp32 parameters -> BF16 GEMM operands."""
        self._ok(self.lib.cf_mlp_pack(self._s(), self.view("W1").data_ptr(), self.view("W2").data_ptr(),
                                      self.view("W3T").data_ptr(), self.W1b.data_ptr(), self.W2b.data_ptr(),
                                      self.W3b.data_ptr(), self.W2T.data_ptr(), self.W3p.data_ptr()),
                 "cf_mlp_pack")

    def gemm(self, A, B, M, N, K, epi, bias, out, zout, ldo):
        rc = self.lib.cf_gemm_bf16(self._s(), A.data_ptr(), B.data_ptr(), M, N, K, epi,
                                   None if bias is None else bias.data_ptr(), out.data_ptr(),
                                   None if zout is None else zout.data_ptr(), ldo, self.err.data_ptr())
        self._ok(rc, "cf_gemm_bf16")

    def gemm_wgrad(self, A, B, M, N, K, out):
        """out[M x N] (FP32) = A B^T with the reduction over K (rows) split
        so that about two waves of CTAs run (cf_gemm_bf16_splitk)."""
        bn = next(c for c in (256, 128, 64, 32, 16) if N % c == 0)
        tiles = (M // 128) * (N // bn)
        splits = max(1, min(K // 64, -(-2 * self.sms // tiles), WGRAD_PARTIAL // (M * N)))
        rc = self.lib.cf_gemm_bf16_splitk(self._s(), A.data_ptr(), B.data_ptr(), M, N, K, splits,
                                          self.wpart.data_ptr(), out.data_ptr(), self.err.data_ptr())
        self._ok(rc, "cf_gemm_bf16_splitk")

    def check_device(self):
        if int(self.err.item()):
            raise RuntimeError("a tensor-core GEMM wait ran out on the device")

    # -- network ----------------------------------------------------------
    def forward(self, Mpad: int, keep: bool = True):
        """Y = MLP(X[:Mpad]); ``keep`` stores the hidden pre-activations
        for backward (at most the training batch)."""
        if keep and Mpad > self.tcap:
            raise ValueError(f"{Mpad} rows exceed the training batch {self.tcap}")
        b1, b2, b3 = self.view("b1"), self.view("b2"), self.view("b3")
        self.gemm(self.X, self.W1b, Mpad, H, K1, EPI_SILU, b1, self.H1, self.Z1 if keep else None, H)
        self.gemm(self.H1, self.W2b, Mpad, H, H, EPI_SILU, b2, self.H2, self.Z2 if keep else None, H)
        self.gemm(self.H2, self.W3b, Mpad, N3, H, EPI_BIAS, b3, self.Y, None, N3)

    def backward(self, M: int, Mpad: int):
        """Gradients of the mean squared error over the first M rows into self.g."""
        s = self._s()
        self._ok(self.lib.cf_mlp_loss_grad(s, self.Y.data_ptr(), self.T.data_ptr(), M, Mpad, self.dY.data_ptr(),
                                           self.dYT.data_ptr(), self.partial.data_ptr()), "cf_mlp_loss_grad")
        # activation gradients
        self.gemm(self.dY, self.W3p, Mpad, H, K3, EPI_F32, None, self.dH, None, H)
        self._ok(self.lib.cf_mlp_silu_bwd(s, self.dH.data_ptr(), self.Z2.data_ptr(), Mpad, self.dZ2.data_ptr(),
                                          self.dZ2T.data_ptr()), "cf_mlp_silu_bwd")
        self.gemm(self.dZ2, self.W2T, Mpad, H, H, EPI_F32, None, self.dH, None, H)
        self._ok(self.lib.cf_mlp_silu_bwd(s, self.dH.data_ptr(), self.Z1.data_ptr(), Mpad, self.dZ1.data_ptr(),
                                          self.dZ1T.data_ptr()), "cf_mlp_silu_bwd")
        # weight gradients: reductions over the rows as K of the GEMM
        for src, dst, cols in ((self.H2, self.H2T, H), (self.H1, self.H1T, H), (self.X, self.XT, K1)):
            self._ok(self.lib.cf_transpose_bf16(s, src.data_ptr(), Mpad, cols, dst.data_ptr()), "cf_transpose_bf16")
        self.gemm_wgrad(self.H2T, self.dYT, H, N3, Mpad, self.view("W3T", self.g))
        self.gemm_wgrad(self.dZ2T, self.H1T, H, H, Mpad, self.view("W2", self.g))
        self.gemm_wgrad(self.dZ1T, self.XT, H, K1, Mpad, self.view("W1", self.g))
        for src, name, cols in ((self.dZ1, "b1", H), (self.dZ2, "b2", H)):
            self._ok(self.lib.cf_colsum_bf16(s, src.data_ptr(), Mpad, cols, self.view(name, self.g).data_ptr()),
                     "cf_colsum_bf16")
        db3 = self.torch.zeros(K3, dtype=self.torch.float32, device="cuda")
        self._ok(self.lib.cf_colsum_bf16(s, self.dY.data_ptr(), Mpad, K3, db3.data_ptr()), "cf_colsum_bf16")
        self.view("b3", self.g).copy_(db3[:N3])

    def loss(self, Mpad: int) -> float:
        part = self.partial[: (Mpad // 256) * 6].view(-1, 6)
        return float(part[:, 0].sum().item())

    def step(self, M: int, Mpad: int) -> float:
        """One Adam step on the rows loaded in X / T; returns the loss."""
        self.forward(Mpad)
        self.backward(M, Mpad)
        self.t += 1
        self._ok(self.lib.cf_adam(self._s(), self.p.data_ptr(), self.g.data_ptr(), self.m.data_ptr(),
                                  self.v.data_ptr(), NPARAM, self.lr, 0.9, 0.999, 1e-8, self.t), "cf_adam")
        self.pack()
        return self.loss(Mpad) / (M * OUT)

    # -- data ---------------------------------------------------------------
    def set_scale(self, grid, Un, Unm1, Unm2):
        """Per-variable scaling: interior RMS of the first and second time
        differences U^n - U^(n-1) and U^n - 2 U^(n-1) + U^(n-2) (10 values)."""
        rms = np.zeros(10)
        arr = (C.c_void_p * 15)(*[t.data_ptr() for t in list(Un) + list(Unm1) + list(Unm2)])
        self._ok(self.lib.cf_mlp_rms(self._s(), grid.X_out, grid.Y_out, grid.Z_out, arr,
                                     self.rms_partial.data_ptr(), 512, rms.ctypes.data), "cf_mlp_rms")
        rms = np.where(rms > 0, rms, 1.0)
        self.scale.copy_(self.torch.from_numpy(rms.astype(np.float32)))
        return rms

    def load_features(self, grid, Un, Unm1, Unm2, rows=None, M=None):
        M = grid.cells if rows is None else len(rows)
        Mpad = _pad(M)
        if Mpad > self.cap:
            raise ValueError(f"{M} rows exceed the capacity {self.cap}")
        arr = (C.c_void_p * 15)(*[t.data_ptr() for t in list(Un) + list(Unm1) + list(Unm2)])
        if rows is None:
            # every cell: the time differences once per array index, then the rows
            n = 10 * (grid.X_out + 6) * (grid.Y_out + 4) * (grid.Z_out + 4)
            if self.D is None or self.D.numel() < n:
                self.D = self.torch.empty(n, dtype=self.torch.float32, device="cuda")
            self._ok(self.lib.cf_mlp_features_grid(self._s(), grid.X_out, grid.Y_out, grid.Z_out, arr,
                                                   self.scale.data_ptr(), Mpad, self.D.data_ptr(), self.X.data_ptr()),
                     "cf_mlp_features_grid")
            return M, Mpad
        self._ok(self.lib.cf_mlp_features(self._s(), grid.X_out, grid.Y_out, grid.Z_out, arr,
                                          self.scale.data_ptr(), None if rows is None else rows.data_ptr(),
                                          M, Mpad, self.X.data_ptr()), "cf_mlp_features")
        return M, Mpad

    def load_targets(self, grid, Unp1, Un, Unm1, Unm2, rows=None):
        M = grid.cells if rows is None else len(rows)
        Mpad = _pad(M)
        if Mpad > self.tcap:
            raise ValueError(f"{M} rows exceed the training batch {self.tcap}")
        arr = (C.c_void_p * 20)(*[t.data_ptr() for t in list(Unp1) + list(Un) + list(Unm1) + list(Unm2)])
        self._ok(self.lib.cf_mlp_targets(self._s(), grid.X_out, grid.Y_out, grid.Z_out, arr, self.coef.ctypes.data,
                                         self.scale.data_ptr(),
                                         self.oscale.data_ptr(), None if rows is None else rows.data_ptr(), M, Mpad,
                                         self.T.data_ptr()), "cf_mlp_targets")
        return M, Mpad

    def _base_sums(self, grid, history, n):
        """sums30 of cf_mlp_base_sums for window n of a history, as (5, 6)."""
        sums = np.zeros(30)
        lv = [history[n + 1], history[n], history[n - 1], history[n - 2]]
        arr = (C.c_void_p * 20)(*[t.data_ptr() for level in lv for t in level])
        self._ok(self.lib.cf_mlp_base_sums(self._s(), grid.X_out, grid.Y_out, grid.Z_out, arr,
                                           self.rms_partial.data_ptr(), 512, sums.ctypes.data), "cf_mlp_base_sums")
        return sums.reshape(5, 6)

    def fit_output_scale(self, grid, history, windows=None, fit_predictor: bool = True):
        """Least-squares coefficients a_v, b_v of the predictor over the
        windows n (default all) of a history [U^0, U^1, ...] of FP64 states
        (``fit_predictor``; else the coefficients are kept), and the
        per-variable output factor: RMS of the predictor's error over the
        RMS of the second time difference, averaged over the windows."""
        wins = list(range(2, len(history) - 1)) if windows is None else list(windows)
        S = [self._base_sums(grid, history, n) for n in wins]
        if fit_predictor and S:
            tot = np.sum(S, axis=0)
            for v in range(5):
                s11, s12, s22, r1, r2, _ = tot[v]
                det = s11 * s22 - s12 * s12
                if det > 1e-12 * max(s11 * s22, 1e-300):
                    self.coef[v] = (r1 * s22 - r2 * s12) / det
                    self.coef[5 + v] = (s11 * r2 - s12 * r1) / det
                else:
                    self.coef[v] = r1 / s11 if s11 > 0 else 0.0
                    self.coef[5 + v] = 0.0
        a, b = self.coef[:5], self.coef[5:]
        r = []
        for s in S:
            s11, s12, s22, r1, r2, tt = s.T
            err = tt - 2 * a * r1 - 2 * b * r2 + a * a * s11 + 2 * a * b * s12 + b * b * s22
            r.append(np.sqrt(np.maximum(err, 0) / np.where(s22 > 0, s22, 1.0)))
        f = np.mean(r, axis=0) if r else np.ones(5)
        f = np.where(f > 0, f, 1.0)
        self.oscale.copy_(self.torch.from_numpy(f.astype(np.float32)))
        self.ogain.copy_(self.oscale)
        return f

    def _rows(self, grid, batch, gen):
        if batch is None or batch >= grid.cells:
            return None
        torch = self.torch
        return torch.randint(0, grid.cells, (batch,), generator=gen, device="cuda", dtype=torch.int32)

    def train(self, grid, history, epochs: int = 20, batch: int | None = None, seed: int = 0,
              holdout: bool = True):
        """Adam on the (U^(n-2), U^(n-1), U^n) -> U^(n+1) windows of a
        history of FP64 states, one step per window and epoch: on all cells
        (``batch`` None) or on ``batch`` cells drawn at random each step.
        With ``holdout`` (and at least two windows) the last window is kept
        out of training and used by ``calibrate``."""
        torch = self.torch
        windows = list(range(2, len(history) - 1))
        if not windows:
            raise ValueError("training needs a history of at least four states")
        val = windows.pop() if holdout and len(windows) >= 2 else None
        self.fit_output_scale(grid, history, windows)
        scales = {n: self.set_scale(grid, history[n], history[n - 1], history[n - 2]).astype(np.float32)
                  for n in windows}
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed)
        losses = []
        for _ in range(epochs):
            for n in windows:
                self.scale.copy_(torch.from_numpy(scales[n]))
                rows = self._rows(grid, batch, gen)
                M, Mpad = self.load_features(grid, history[n], history[n - 1], history[n - 2], rows=rows)
                self.load_targets(grid, history[n + 1], history[n], history[n - 1], history[n - 2], rows=rows)
                losses.append(self.step(M, Mpad))
        self.check_device()
        self.validation = None
        if val is not None:
            self.validation = self.calibrate(grid, history[val + 1], history[val], history[val - 1],
                                             history[val - 2], batch=batch, seed=seed + 1)
        return losses

    def calibrate(self, grid, Unp1, Un, Unm1, Unm2, batch: int | None = None, seed: int | None = None):
        """Least-squares gain per output of the correction on a window the
        network has not been trained on, alpha_v = <t, y> / <y, y> clipped
        to [0, 2]; the guess then uses oscale * alpha, so that a correction
        that does not reduce the extrapolation error there is scaled down.
        Returns alpha and the window's RMS error of predictor +
        correction relative to the predictor alone, per variable, before
        and after the gain (keys ``err_over_extrapolation*``: the predictor
        is the fitted one)."""
        torch = self.torch
        gen = self.gen
        if seed is not None:
            gen = torch.Generator(device="cuda")
            gen.manual_seed(seed)
        self.set_scale(grid, Un, Unm1, Unm2)
        rows = self._rows(grid, batch if batch is not None else self.tcap, gen)
        M, Mpad = self.load_features(grid, Un, Unm1, Unm2, rows=rows)
        self.load_targets(grid, Unp1, Un, Unm1, Unm2, rows=rows)
        self.forward(Mpad, keep=False)
        sums = np.zeros(15)
        self._ok(self.lib.cf_mlp_dot(self._s(), self.Y.data_ptr(), self.T.data_ptr(), M, self.rms_partial.data_ptr(),
                                     128, sums.ctypes.data), "cf_mlp_dot")
        ty, yy, tt = sums[:5], sums[5:10], sums[10:]
        tt = np.where(tt > 0, tt, 1.0)
        alpha = np.clip(np.where(yy > 0, ty / np.where(yy > 0, yy, 1.0), 0.0), 0.0, 2.0)
        before = np.sqrt(np.maximum(tt - 2 * ty + yy, 0) / tt)
        after = np.sqrt(np.maximum(tt - 2 * alpha * ty + alpha * alpha * yy, 0) / tt)
        self.ogain.copy_(self.oscale * torch.from_numpy(alpha.astype(np.float32)).to(self.oscale.device))
        return {"alpha": alpha.tolist(), "err_over_extrapolation_raw": before.tolist(),
                "err_over_extrapolation": after.tolist()}

    def update(self, grid, Unp1, Un, Unm1, Unm2, adam_steps: int = 2, batch: int = 65536):
        """Online step once U^(n+1) is known: first the gain on this window
        (which the network has not seen, so the fit is out of sample), then
        ``adam_steps`` Adam steps on random cells of it.  Returns the
        calibration of ``calibrate``."""
        cal = self.calibrate(grid, Unp1, Un, Unm1, Unm2, batch=batch)
        for _ in range(adam_steps):
            rows = self._rows(grid, batch, self.gen)
            M, Mpad = self.load_features(grid, Un, Unm1, Unm2, rows=rows)
            self.load_targets(grid, Unp1, Un, Unm1, Unm2, rows=rows)
            self.step(M, Mpad)
        self.updates.append(cal)
        return cal

    @staticmethod
    def extrapolate(grid, Un, Unm1, Unm2, out, stream=None):
        """out (U_) = U^n + 2 dU^n - dU^(n-1) on every interior cell."""
        import torch
        lib = _lib.load()
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        a = (C.c_void_p * 15)(*[t.data_ptr() for t in list(Un) + list(Unm1) + list(Unm2)])
        o = (C.c_void_p * 5)(*[t.data_ptr() for t in out])
        rc = lib.cf_mlp_apply(s, grid.X_out, grid.Y_out, grid.Z_out, a, None, None, None, None, o)
        if rc != _lib.CF_OK:
            raise RuntimeError(f"cf_mlp_apply failed with status {rc}")

    def set_scale_device(self, grid, Un, Unm1, Unm2):
        """The scales of ``set_scale`` computed and stored on the device,
        stream-ordered (no host round trip)."""
        arr = (C.c_void_p * 15)(*[t.data_ptr() for t in list(Un) + list(Unm1) + list(Unm2)])
        self._ok(self.lib.cf_mlp_scale(self._s(), grid.X_out, grid.Y_out, grid.Z_out, arr,
                                       self.rms_partial.data_ptr(), 512, self.scale.data_ptr()), "cf_mlp_scale")

    def guess(self, grid, Un, Unm1, Unm2, out):
        """out (U_) = U^n + a dU^n + b d2U + the network's correction on
        every interior cell; the grid's cells must fit the capacity."""
        self.set_scale_device(grid, Un, Unm1, Unm2)
        M, Mpad = self.load_features(grid, Un, Unm1, Unm2)
        self.forward(Mpad, keep=False)
        a = (C.c_void_p * 15)(*[t.data_ptr() for t in list(Un) + list(Unm1) + list(Unm2)])
        o = (C.c_void_p * 5)(*[t.data_ptr() for t in out])
        self._ok(self.lib.cf_mlp_apply(self._s(), grid.X_out, grid.Y_out, grid.Z_out, a, self.coef.ctypes.data,
                                       self.scale.data_ptr(),
                                       self.ogain.data_ptr(), self.Y.data_ptr(), o), "cf_mlp_apply")

"""Physical time steps with an initial guess for the pseudo-time iterations.

``Stepper`` drives ``Context.step`` (the C-ABI ``cf_step``: sub-iterations
of the dual-time LU-SGS to a residual tolerance) and keeps the last three
time levels U^n, U^(n-1), U^(n-2) on the device, so that each step can start
its sub-iterations from

* ``None``: U^n (the reference's start, main.cpp:443-462),
* ``"extrapolate"``: the quadratic extrapolation U^n + 2 dU^n - dU^(n-1),
* a trained ``mlp.LearnedGuess``: that extrapolation corrected by the
  network.

The tolerance and the iteration loop are the same in every case; only the
starting point differs.  With ``online`` set, a learned guess also learns
during the run: once a step has converged, the network's gain is refitted
on that step (which it predicted without seeing it) and it takes a few Adam
steps on it (``LearnedGuess.update``).  Both guesses replace the interior
cells of U_; its ghost cells are rebuilt by the boundary conditions at the
start of every sub-iteration, as in the plain loop.
"""
from __future__ import annotations

from collections import deque

from . import mlp


class Stepper:
    def __init__(self, ctx, fields: dict, online: dict | None = None, **step_kw):
        self.ctx = ctx
        self.f = fields
        self.online = online
        # a new run: the residual maxima start over, and the metric arrays
        # are fixed for the run (the FP32 path keeps FP32 copies of them)
        ctx.step_reset()
        step_kw.setdefault("static_metrics", True)
        self.kw = step_kw
        self.n = 0
        self.hist = deque(maxlen=3)
        self.hist.append([u.clone() for u in fields["U"]])

    def restore(self, levels, step: int = 0):
        """Restart from saved time levels [..., U^(n-1), U^n] (the last
        three are kept): U_ = U = U^n, Uq = U^(n-1)."""
        self.hist.clear()
        for lv in levels[-3:]:
            self.hist.append([u.clone() for u in lv])
        un = self.hist[-1]
        uq = self.hist[-2] if len(self.hist) > 1 else un
        for v in range(5):
            self.f["U_"][v].copy_(un[v])
            self.f["U"][v].copy_(un[v])
            self.f["Uq"][v].copy_(uq[v])
        self.n = step

    def step(self, guess=None):
        """One physical step; returns (sub-iterations, er[5], Q)."""
        if guess is not None and len(self.hist) == 3:
            un, u1, u2 = self.hist[2], self.hist[1], self.hist[0]
            if isinstance(guess, str):
                if guess != "extrapolate":
                    raise ValueError(f"unknown guess {guess!r}")
                mlp.LearnedGuess.extrapolate(self.ctx.grid, un, u1, u2, self.f["U_"])
            else:
                guess.guess(self.ctx.grid, un, u1, u2, self.f["U_"])
        self.n += 1
        it, er, q = self.ctx.step(self.f, step=self.n, **self.kw)
        if self.online is not None and guess is not None and not isinstance(guess, str) and len(self.hist) == 3:
            guess.update(self.ctx.grid, self.f["U"], self.hist[2], self.hist[1], self.hist[0], **self.online)
        self.hist.append([u.clone() for u in self.f["U"]])
        return it, er, q

    def history(self):
        return list(self.hist)


def fields_from_workload(w, torch, grid):
    """cf_fields of a bench.DeviceWorkload-like object (state U = U_ = Uq)."""
    z = lambda: torch.zeros(grid.shape, dtype=torch.float64, device="cuda")
    return {"U_": w.U, "U": [u.clone() for u in w.U], "Uq": [u.clone() for u in w.U], "J": w.J, "Y_point": w.Yp,
            "cell_metric": w.cm, "face_J": [w.fu[0], w.fv[0], w.fw[0]],
            "face_metric": [w.fu[1:], w.fv[1:], w.fw[1:]], "Ep": w.Ep, "inF": [w.Fx, w.Fy, w.Fz], "vF": w.vF,
            "LL": w.LL, "ML": w.ML, "MR": [z() for _ in range(5)], "NR": [z() for _ in range(5)],
            "NL": [z() for _ in range(5)], "Residual": [z() for _ in range(5)]}

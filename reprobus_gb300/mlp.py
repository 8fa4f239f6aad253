"""The network of the Newton solvers' learned restart (libreprobus_gb300.so,
mlp_kernels.cu): a 64-256-256-256-64 MLP with SiLU, BF16 weights and
activations and FP32 accumulation on the tcgen05 tensor cores, trained on
the GPU by the library's own forward/backward kernels on cells that the plain
FP64 Newton solver integrates.

The network corrects the solvers' plain start (npass reference passes from
the start state); a solver uses the corrected start for the cells whose
plain start misses the convergence test. Features of a cell (64, raw): log10 of the 42 transported and
15 short-lived mixing ratios of the plain start (floored at 1e-30), T, ln p,
cos(sza), log10 aerosol surface area (floored at 1e-12), latitude, time of
day, 0. Targets (64, raw): log10 of the ratio of each of the 57 end-of-step
mixing ratios to its plain-start value (floored the same way), 7 zero
columns. The network learns normalised units; the normalisation (means and
standard deviations of the training set) travels with the weights.

torch supplies device memory only; all computation runs in the library.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import chem

NFEAT = 64
NOUT = 64
NY = 57
DIMS = [(64, 256), (256, 256), (256, 256), (256, 64)]  # (fan_in, fan_out) per layer
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "mlp_warmstart.npz")
YCLIP = 2.0  # largest log10 correction learned (a factor of 100)


def nparams():
    return sum(i * o + o for i, o in DIMS)


def unpack(params):
    """[(W (fan_out x fan_in), b)] from the packed FP32 vector."""
    out, o = [], 0
    for i, n in DIMS:
        W = params[o:o + i * n].reshape(n, i)
        o += i * n
        b = params[o:o + n]
        o += n
        out.append((W, b))
    return out


class Mlp:
    """One network on the current CUDA device."""

    def __init__(self, batch_cap=8192, seed=0):
        self.lib = chem.load_library()
        h = ctypes.c_void_p()
        chem._check(self.lib.reprobus_mlp_create(int(batch_cap), int(seed), ctypes.byref(h)))
        self.handle = h.value
        self.batch_cap = batch_cap
        assert self.lib.reprobus_mlp_nparams() == nparams()

    def close(self):
        if getattr(self, "handle", None):
            self.lib.reprobus_mlp_free(ctypes.c_void_p(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _fp(a):
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if a is not None else None

    def set_params(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        chem._check(self.lib.reprobus_mlp_set_params(ctypes.c_void_p(self.handle), self._fp(p), self._fp(n)))

    def get_params(self):
        p = np.zeros(nparams(), np.float32)
        n = np.zeros(2 * NFEAT + 3 * NOUT, np.float32)
        chem._check(self.lib.reprobus_mlp_get_params(ctypes.c_void_p(self.handle), self._fp(p), self._fp(n)))
        return p, n

    def train_step(self, X, Y, lr, stream=None):
        """One Adam step on device batches X, Y (float32 CUDA tensors B x 64);
        returns the loss before the step."""
        loss = np.zeros(1, np.float32)
        chem._check(self.lib.reprobus_mlp_train_step(ctypes.c_void_p(self.handle), chem._dp(X), chem._dp(Y),
                                                     int(X.shape[0]), float(lr), self._fp(loss),
                                                     ctypes.c_void_p(stream)))
        return float(loss[0])

    def grads(self, X, Y):
        g = np.zeros(nparams(), np.float32)
        loss = np.zeros(1, np.float32)
        chem._check(self.lib.reprobus_mlp_grads(ctypes.c_void_p(self.handle), chem._dp(X), chem._dp(Y),
                                                int(X.shape[0]), self._fp(g), self._fp(loss), None))
        return g, float(loss[0])

    def forward(self, X, Y):
        """Y = network(X) on the tensor cores (any number of rows)."""
        chem._check(self.lib.reprobus_mlp_forward(ctypes.c_void_p(self.handle), chem._dp(X), chem._dp(Y),
                                                  int(X.shape[0]), None))

    def set_wait_limit(self, polls=-1):
        """Polls after which the inference kernel's waits give up (-1: the
        default; 0: at once). A fault-handling hook: a wait that gives up
        makes forward() and a step with the learned restart raise REPROBUS_ERR_TIMEOUT
        and leaves the network usable."""
        chem._check(self.lib.reprobus_mlp_set_wait_limit(ctypes.c_void_p(self.handle), int(polls)))

    def save(self, path):
        p, n = self.get_params()
        np.savez(path, params=p, norm=n)

    def load(self, path=WEIGHTS):
        z = np.load(path)
        self.set_params(z["params"], z["norm"])


def cell_states(dc, case):
    """Start (or current) mixing ratios of the 57 unknowns of every chemistry
    cell, as a CUDA tensor ncell x 57 (cells in the diagnostics order)."""
    nc = case.nlon * case.nlat * case.nivbas
    q = dc["qj1"].view(43, -1)[:42, :nc]
    h = dc["hc"].view(15, -1)[:, :nc]
    import torch
    return torch.cat([q, h], 0).T


def sample(case, solver=chem.SOLVER_NEWTON64, npass=5):
    """(features, targets) of every chemistry cell of a case: the features of
    the plain start (npass reference passes), and the log10 ratios of the
    end-of-step mixing ratios the plain solver returns (no conserv) to the
    plain-start ones. CUDA float32 tensors ncell x 64."""
    import torch
    from .resident import DeviceCase
    dc = DeviceCase(case)
    nc = case.nlon * case.nlat * case.nivbas
    h = chem.ChemStep.for_case(case, niter=5, flags=0)
    h.set_solver(solver, npass=npass)
    feat = torch.empty(nc, NFEAT, dtype=torch.float32, device="cuda")
    a = dc.args()
    h.features_dev(1, case.nlat, case.daynum, case.dt, a[0], a[1], a[2], a[3], a[4], case.irapp, a[6], a[7], feat)
    h.step_dev(1, case.nlat, case.daynum, case.dt, *a)
    q1 = cell_states(dc, case)
    y = torch.zeros(nc, NOUT, dtype=torch.float32, device="cuda")
    l1 = torch.log10(q1.clamp_min(1e-30))
    l0 = feat[:, :NY].double()
    d = (l1 - l0).clamp(-YCLIP, YCLIP)
    # species below 1e-20 mol/mol at both ends need no correction (the solver's
    # accuracy criterion ignores them)
    d = torch.where(torch.maximum(l1, l0) < -20.0, torch.zeros_like(d), d)
    y[:, :NY] = d.float()
    h.close()
    torch.cuda.synchronize()
    return feat, y


def normalisation(X, Y):
    """Feature and target means / standard deviations (std floored) of a
    training set, packed as the library expects."""
    xm, xs = X.mean(0), X.std(0).clamp_min(1e-3)
    ym, ys = Y.mean(0), Y.std(0).clamp_min(1e-3)
    xm[-1], xs[-1] = 0.0, 1.0
    ym[NY:], ys[NY:] = 0.0, 1.0
    import torch
    return torch.cat([xm, xs, ym, ys, torch.zeros_like(ym)]).cpu().numpy().astype(np.float32)


THRESHOLDS = np.concatenate([[0.0], np.logspace(-4, 0, 17), [np.inf]])


def fit_thresholds(net, X, Y):
    """Per output, the smallest |predicted correction| that is applied
    (out_min), fitted on validation cells (X, Y): the threshold of a grid that
    minimises the mean over cells of log10(1e-4 + |error of the start|), where
    a prediction below the threshold leaves the plain start (error |y|).
    inf switches an output off. Returns the thresholds."""
    import torch
    p, n = net.get_params()
    n = n.copy()
    n[2 * NFEAT + 2 * NOUT:] = 0.0
    net.set_params(None, n)
    P = torch.zeros_like(Y)
    net.forward(X, P)
    tau = np.full(NOUT, np.inf, np.float32)
    for i in range(NY):
        y, e = Y[:, i], P[:, i]
        best, bt = None, np.inf
        for t in THRESHOLDS:
            err = torch.where(e.abs() >= float(t), (e - y).abs(), y.abs())
            score = float(torch.log10(1e-4 + err).mean())
            if best is None or score < best - 1e-6:
                best, bt = score, t
        tau[i] = bt
    n[2 * NFEAT + 2 * NOUT:] = np.where(np.isfinite(tau), tau, 3.0e38)
    net.set_params(None, n)
    return tau


def train(net, X, Y, steps, batch=8192, lr=1e-3, lr_end=1e-5, seed=0, log_every=0):
    """Adam on random batches of the device training set (cosine-decayed
    learning rate); returns the loss history."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    n = X.shape[0]
    hist = []
    for s in range(steps):
        idx = torch.randint(0, n, (batch,), device="cuda", generator=g)
        lr_s = lr_end + 0.5 * (lr - lr_end) * (1 + np.cos(np.pi * s / max(steps - 1, 1)))
        loss = net.train_step(X[idx].contiguous(), Y[idx].contiguous(), lr_s)
        hist.append(loss)
        if log_every and s % log_every == 0:
            print(f"step {s} lr {lr_s:.2e} loss {loss:.5f}", flush=True)
    return hist

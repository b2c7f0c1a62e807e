"""The learned surrogate of the forward model and the surrogate-assisted
inverse solver.

Surrogate: MLP (ln mu_a, ln mu_s', g, d, n) -> means and log-variances of
(R_d, T_d, T_u) for a slab between n=1.5 / 0.1 cm slides in the two-sphere
geometry of the benchmark set (5.08 cm spheres, 1.27/1.27/0.635 cm ports, wall
0.98, crosstalk on).  Training data come from the batched Monte Carlo (one
persistent launch per chunk of samples); the network is trained on the GPU by
libismc's own tcgen05 BF16 GEMM forward/backward and Adam kernels
(ismc_mlp_* in include/ismc.h).

Inverse solver (surrogate path): for measurements (R_d, T_d, T_u) with noise
sigma, (1) a grid search of the surrogate over (ln mu_a, ln mu_s') proposes a
start, (2) Gauss-Newton steps on the surrogate refine it, (3) one Monte Carlo
run at the answer verifies it, and (4) the solve falls back to the plain path
(PRAXIS on Monte Carlo, ismc_solve_batch) when the verified values miss the
measurement by more than 3 sigma.  Everything is batched over measurements.
"""
import ctypes as C
import math
import time

import numpy as np

from .api import (IsmcError, Layer, load_library, make_solve, slab_instances,
                  tallies_mean_se)
from .workloads import bench_spheres

LO = np.array([math.log(0.01), math.log(1.0), 0.6, 0.02, 1.33])
HI = np.array([math.log(10.0), math.log(100.0), 0.95, 0.5, 1.5])


def sample_stack(mua, musr, g, d, n):
    """The surrogate's forward-model geometry: slab between n=1.5, 0.1 cm slides."""
    return [Layer.slide(1.5, 0.1), Layer.from_reduced(n, mua, musr, g, d), Layer.slide(1.5, 0.1)]


def sample_inputs(n, seed=42):
    """Uniform samples in (ln mu_a, ln mu_s', g, d, n)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return (LO + (HI - LO) * rng.random((n, 5))).astype(np.float64)


def simulate(engine, X, n_packets, seed=42, chunk=65536, spheres=None, mode="compat"):
    """Monte Carlo targets for input rows X: returns (Y means [n x 3], SE [n x 3])
    of (R_d, T_d, T_u), one batched launch per chunk of rows; row i runs
    sample_stack(exp X[i,0], exp X[i,1], X[i,2], X[i,3], X[i,4]) on Philox
    stream i."""
    sph = spheres or bench_spheres()
    X = np.asarray(X, dtype=np.float64)
    Y = np.empty((len(X), 3))
    S = np.empty((len(X), 3))
    for a in range(0, len(X), chunk):
        rows = X[a:a + chunk]
        insts = slab_instances(np.exp(rows[:, 0]), np.exp(rows[:, 1]), rows[:, 2], rows[:, 3],
                               rows[:, 4], sph, n_packets, seed=seed, stream0=a, mode=mode)
        mean, se, _ = tallies_mean_se(engine.run_batch_raw(insts))
        Y[a:a + len(rows)] = mean[:, [1, 3, 4]]
        S[a:a + len(rows)] = se[:, [1, 3, 4]]
    return Y, S


class Surrogate:
    """Handle of an on-GPU MLP (ismc_mlp_*)."""

    def __init__(self, device=0, max_batch=4096, seed=42):
        import torch
        self.torch = torch
        self.lib = load_library()
        self.h = C.c_void_p()
        rc = self.lib.ismc_mlp_create(device, max_batch, seed, C.byref(self.h))
        if rc:
            raise IsmcError(rc, self._err(None))
        self.device = device
        self.max_batch = max_batch
        self.nparam = int(self.lib.ismc_mlp_nparam())

    def _err(self, h):
        buf = C.create_string_buffer(512)
        if h:
            self.lib.ismc_mlp_last_error(h, buf, 512)
        else:
            self.lib.ismc_last_error(None, buf, 512)
        return buf.value.decode(errors="replace")

    def _check(self, rc):
        if rc:
            raise IsmcError(rc, self._err(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.ismc_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- parameters
    def get_params(self):
        p = np.empty(self.nparam, dtype=np.float32)
        self._check(self.lib.ismc_mlp_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)),
                                                  self.nparam))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self.lib.ismc_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)),
                                                  self.nparam))

    # -- device tensors in, device tensors out
    def _dev(self, a, cols):
        t = self.torch
        if not isinstance(a, t.Tensor):
            a = t.as_tensor(np.asarray(a, dtype=np.float32))
        a = a.to(device=f"cuda:{self.device}", dtype=t.float32).contiguous()
        assert a.ndim == 2 and a.shape[1] == cols
        # the library's stream must not read before torch's producer finished
        t.cuda.current_stream(a.device).synchronize()
        return a

    def forward(self, x):
        """Outputs [n x 6] (mu R_d, T_d, T_u, log-var R_d, T_d, T_u) for inputs [n x 5];
        rows are padded to a multiple of 128 and processed in max_batch slices."""
        t = self.torch
        x = self._dev(x, 5)
        n = x.shape[0]
        out = t.empty((n, 6), device=x.device, dtype=t.float32)
        for a in range(0, n, self.max_batch):
            xb = x[a:a + self.max_batch]
            nb = xb.shape[0]
            pad = (-nb) % 128
            if pad:
                xb = t.cat([xb, xb[-1:].expand(pad, 5)], 0).contiguous()
            ob = t.empty((xb.shape[0], 6), device=x.device, dtype=t.float32)
            self._check(self.lib.ismc_mlp_forward(self.h, xb.data_ptr(), xb.shape[0], ob.data_ptr()))
            out[a:a + nb] = ob[:nb]
        return out

    def grad(self, x, y):
        """(loss, flat fp32 gradient) of the mean Gaussian NLL on one batch."""
        t = self.torch
        x, y = self._dev(x, 5), self._dev(y, 3)
        g = t.empty(self.nparam, device=x.device, dtype=t.float32)
        loss = C.c_float()
        self._check(self.lib.ismc_mlp_grad(self.h, x.data_ptr(), y.data_ptr(), x.shape[0],
                                           g.data_ptr(), C.byref(loss)))
        return loss.value, g.cpu().numpy()

    def train_step(self, x, y, lr, want_loss=False):
        loss = C.c_float()
        self._check(self.lib.ismc_mlp_train_step(self.h, x.data_ptr(), y.data_ptr(), x.shape[0],
                                                 float(lr), C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def train(self, X, Y, epochs=20, batch=4096, lr=1e-3, seed=42, log_every=0):
        """Adam with cosine-decayed learning rate over `epochs` passes of (X, Y)
        (device or host arrays).  Returns the per-epoch mean losses."""
        t = self.torch
        X, Y = self._dev(X, 5), self._dev(Y, 3)
        n = X.shape[0] // batch * batch
        steps_per_epoch = n // batch
        total = epochs * steps_per_epoch
        g = t.Generator(device=X.device)
        g.manual_seed(seed)
        hist = []
        step = 0
        for ep in range(epochs):
            perm = t.randperm(X.shape[0], generator=g, device=X.device)[:n]
            Xs, Ys = X[perm].contiguous(), Y[perm].contiguous()
            t.cuda.current_stream(X.device).synchronize()       # gather done before use
            lrs = np.array([0.5 * lr * (1 + math.cos(math.pi * (step + b) / total))
                            for b in range(steps_per_epoch)], dtype=np.float32)
            loss = C.c_float()
            # the whole epoch in one native call: no per-step Python
            self._check(self.lib.ismc_mlp_train_epoch(
                self.h, Xs.data_ptr(), Ys.data_ptr(), n, batch,
                lrs.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)))
            step += steps_per_epoch
            hist.append(float(loss.value))
        return hist


# ----------------------------------------------------------------------------
# surrogate-assisted inverse solve
# ----------------------------------------------------------------------------
def _grid(nmua=48, nmus=48):
    a = np.linspace(LO[0], HI[0], nmua)
    s = np.linspace(LO[1], HI[1], nmus)
    A, S = np.meshgrid(a, s, indexing="ij")
    return np.stack([A.ravel(), S.ravel()], 1)


def _gauss_newton(sur, x, meas, w, offset, steps, g, d, n, h=0.05):
    """Damped Gauss-Newton on the surrogate for rows x [m x 2] (ln mu_a, ln mu_s'):
    minimise sum_k (w_k (meas_k - f_k(x) - offset_k))^2 with central
    differences of step h (the network is piecewise smooth at bf16 activation
    resolution, so the step is kept well above it).  w is [m x 3] or [3]."""
    w = np.broadcast_to(np.asarray(w, dtype=np.float64), meas.shape)
    m = len(x)
    for _ in range(steps):
        pts = np.concatenate([x, x + [h, 0.0], x - [h, 0.0], x + [0.0, h], x - [0.0, h]], 0)
        Xp = np.concatenate([pts, np.tile([g, d, n], (len(pts), 1))], 1)
        o = sur.forward(Xp).cpu().numpy()[:, :3].astype(np.float64)
        f0 = o[:m] + offset
        J = np.stack([(o[m:2 * m] - o[2 * m:3 * m]) / (2 * h),
                      (o[3 * m:4 * m] - o[4 * m:]) / (2 * h)], 2) * w[:, :, None]   # m x 3 x 2
        rsd = (meas - f0) * w                                                         # m x 3
        JtJ = np.einsum("mki,mkj->mij", J, J)
        JtJ = JtJ + (1e-3 * np.trace(JtJ, axis1=1, axis2=2)[:, None, None] + 1e-9) * np.eye(2)
        Jtr = np.einsum("mki,mk->mi", J, rsd)
        dx = np.linalg.solve(JtJ, Jtr[..., None])[..., 0]
        dx = np.clip(dx, -0.5, 0.5)
        x = np.clip(x + dx, LO[:2], HI[:2])
    return x


def _verify(engine, x, g, d, n, packets, seed, stream0=0):
    insts = slab_instances(np.exp(x[:, 0]), np.exp(x[:, 1]), g, d, n, bench_spheres(), packets,
                           seed=seed, stream0=stream0)
    mean, se, _ = tallies_mean_se(engine.run_batch_raw(insts))
    return mean[:, [1, 3, 4]], se[:, [1, 3, 4]]


def objective_weights(meas, sigma, objective="chi2"):
    """Per-measurement residual weights [m x 3] for (R_d, T_d, T_u).

    "chi2": residuals in units of the measurement noise sigma, the same
    weighting as the 3-sigma verification test;
    "reference": the plain path's cost (minimization.py:231-238,
    ISMLMC-minimization.cu:120-128): relative residuals of R_d and T_d,
    absolute residual of T_u."""
    meas = np.asarray(meas, dtype=np.float64)
    if objective == "chi2":
        return np.broadcast_to(1.0 / np.asarray(sigma, dtype=np.float64), meas.shape).copy()
    if objective != "reference":
        raise ValueError(f"unknown objective {objective!r}")
    w = np.ones_like(meas)
    w[:, 0] = 1.0 / np.maximum(np.abs(meas[:, 0]), 1e-6)
    w[:, 1] = 1.0 / np.maximum(np.abs(meas[:, 1]), 1e-6)
    return w


def surrogate_solve(sur, engine, meas, sigma, g=0.9, d=0.1, n=1.4, gn_steps=10, verify_packets=300_000,
                    seed=7, fallback=True, correct=True, plain_packets=100_000, plain_max_evals=400,
                    objective="chi2", anchor_packets=0, anchor_steps=5, test=None,
                    fallback_h0=0.15):
    """Solve many measurements [m x 3] of (R_d, T_d, T_u) with noise sigma (3,).

    (1) The surrogate on a 48 x 48 (ln mu_a, ln mu_s') grid proposes a start;
    (2) Gauss-Newton steps on the surrogate refine it.  (2b) With
    `anchor_packets`, every solve is anchored to Monte Carlo: one run of that
    many packets at its point gives the Monte Carlo-minus-surrogate difference
    there, and `anchor_steps` more Gauss-Newton steps minimise on the surrogate
    shifted by it -- the local bias of the network is then gone, and the answer
    approaches the minimum of the Monte Carlo objective itself.  (3) One Monte
    Carlo run of `verify_packets` verifies the final point (3e5 packets: on the
    solve benchmark, 1e6 gave the same answers, fallbacks and accuracy at half
    the speed).  (3b) With
    `correct`, a solve that fails the test is re-anchored at its point by that
    verification, re-solved and verified again.  (4) What still fails falls
    back to the plain path (PRAXIS on Monte Carlo), started from the
    surrogate's answer with PRAXIS's initial step `fallback_h0` (in ln units:
    the answer is already close).

    Steps (1)-(3b) minimise `objective` (see objective_weights).  The test of
    step (3) is `test`: "fit" (the default for chi2) asks every verified value
    to lie within 3 sigma of the measurement, sqrt(sigma^2 + se^2); "surrogate"
    (the default otherwise) asks the surrogate's prediction at the final point,
    anchor offset included, to lie within 3 standard errors of the verifying
    Monte Carlo run.  Returns dict with x [m x 2] (mu_a, mu_s'), the verified
    MC values, masks of corrected and fallback solves, and timings."""
    import torch
    meas = np.asarray(meas, dtype=np.float64)
    sig = np.asarray(sigma, dtype=np.float64)
    wts = objective_weights(meas, sig, objective)
    test = test or ("fit" if objective == "chi2" else "surrogate")
    if test not in ("fit", "surrogate"):
        raise ValueError(f"unknown test {test!r}")
    m = len(meas)
    T = {}

    def predict(x):
        Xi = np.concatenate([x, np.tile([g, d, n], (len(x), 1))], 1)
        return sur.forward(Xi).cpu().numpy()[:, :3].astype(np.float64)

    t0 = time.perf_counter()
    # (1) grid proposal, shared surrogate evaluations for all measurements
    grid = _grid()
    X = np.concatenate([grid, np.tile([g, d, n], (len(grid), 1))], 1)
    ot = sur.forward(X)[:, :3]
    mt = torch.as_tensor(meas, device=ot.device, dtype=torch.float32)
    wt = torch.as_tensor(wts, device=ot.device, dtype=torch.float32)
    best = []
    for a in range(0, m, 4096):
        r = (((ot[None, :, :] - mt[a:a + 4096, None, :]) * wt[a:a + 4096, None, :]) ** 2).sum(-1)
        best.append(r.argmin(1))
    x = grid[torch.cat(best).cpu().numpy()].copy()
    T["propose_s"] = time.perf_counter() - t0
    # (2) Gauss-Newton on the surrogate
    t1 = time.perf_counter()
    x = _gauss_newton(sur, x, meas, wts, 0.0, gn_steps, g, d, n)
    T["gauss_newton_s"] = time.perf_counter() - t1
    # (2b) anchor every solve to Monte Carlo at its point
    t1 = time.perf_counter()
    off = np.zeros_like(meas)
    off_se = np.zeros_like(meas)
    if anchor_packets:
        Va, off_se = _verify(engine, x, g, d, n, anchor_packets, seed + 3, stream0=2 * m)
        off = Va - predict(x)
        x = _gauss_newton(sur, x, meas, wts, off, anchor_steps, g, d, n)
    T["anchor_s"] = time.perf_counter() - t1
    # (3) Monte Carlo verification at the answers: one batched launch
    t2 = time.perf_counter()
    V, VS = _verify(engine, x, g, d, n, verify_packets, seed)
    pred = predict(x) + off
    T["verify_s"] = time.perf_counter() - t2

    def failed(V, VS, pred, pred_se):
        if test == "fit":
            return np.abs(V - meas) > 3 * np.sqrt(sig ** 2 + VS ** 2)
        return np.abs(V - pred) > 3 * np.sqrt(VS ** 2 + pred_se ** 2)

    fails = failed(V, VS, pred, off_se)          # [m x 3]: which of R_d, T_d, T_u failed
    first_fails = fails.sum(0)
    miss = fails.any(1)
    corrected = np.zeros(m, dtype=bool)
    # (3b) re-anchor the failures at their verified values, verify again
    t3 = time.perf_counter()
    if correct and miss.any():
        idx = np.nonzero(miss)[0]
        xi = x[idx]
        oi = V[idx] - predict(xi)
        xi = _gauss_newton(sur, xi, meas[idx], wts[idx], oi, gn_steps, g, d, n)
        Vi, VSi = _verify(engine, xi, g, d, n, verify_packets, seed + 1, stream0=m)
        x[idx], V[idx], VS[idx] = xi, Vi, VSi
        pred[idx] = predict(xi) + oi
        off_se[idx] = VS[idx]
        corrected[idx] = True
        miss = failed(V, VS, pred, off_se).any(1)
    T["correct_s"] = time.perf_counter() - t3
    # (4) fallback to the plain path for what still misses
    t4 = time.perf_counter()
    xr = np.exp(x)
    if fallback and miss.any():
        idx = np.nonzero(miss)[0]
        sph = bench_spheres()
        reqs = [make_solve(sample_stack(1.0, 10.0, g, d, n), 1, sph, plain_packets,
                           (meas[i, 0], None, meas[i, 1], meas[i, 2]), x0=tuple(xr[i]),
                           seed=seed + 1, lo=(0.005, 0.5), hi=(20.0, 200.0),
                           max_evals=plain_max_evals, h0=fallback_h0) for i in idx]
        outp = engine.solve_batch(reqs)
        for i, o in zip(idx, outp):
            xr[i] = (o.x[0], o.x[1])
        fallback_evals = sum(int(o.evals) for o in outp)
    else:
        fallback_evals = 0
    T["fallback_s"] = time.perf_counter() - t4
    T["total_s"] = time.perf_counter() - t0
    # Monte Carlo packets spent: anchors, verification, re-verification, fallback objectives
    mc = (m * (1 if anchor_packets else 0)) * anchor_packets + \
        (m + int(corrected.sum())) * verify_packets + fallback_evals * plain_packets
    return {"x": xr, "verified": V, "verified_se": VS, "corrected": corrected, "fallback": miss,
            "timing": T, "mc_packets": mc, "fallback_evals": fallback_evals,
            "objective": objective, "test": test, "anchor_packets": anchor_packets,
            "first_test_failures": first_fails.tolist()}

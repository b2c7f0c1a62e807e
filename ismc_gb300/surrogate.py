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

from . import _abi
from .api import Engine, IsmcError, Layer, load_library, make_instance, make_solve
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
    of (R_d, T_d, T_u), one batched launch per chunk of rows."""
    sph = spheres or bench_spheres()
    Y = np.empty((len(X), 3))
    S = np.empty((len(X), 3))
    for a in range(0, len(X), chunk):
        rows = X[a:a + chunk]
        insts = [make_instance(sample_stack(math.exp(r[0]), math.exp(r[1]), r[2], r[3], r[4]),
                               sph, n_packets, seed=seed, stream=a + i, mode=mode)
                 for i, r in enumerate(rows)]
        res = engine.run_batch(insts)
        for i, t in enumerate(res):
            Y[a + i] = (t.mean[1], t.mean[3], t.mean[4])
            S[a + i] = (t.se[1], t.se[3], t.se[4])
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
            losses = []
            for b in range(steps_per_epoch):
                cur = 0.5 * lr * (1 + math.cos(math.pi * step / total))
                want = (b == steps_per_epoch - 1) or (log_every and b % log_every == 0)
                l = self.train_step(Xs[b * batch:(b + 1) * batch], Ys[b * batch:(b + 1) * batch],
                                    cur, want_loss=want)
                if want:
                    losses.append(l)
                step += 1
            hist.append(float(np.mean(losses)))
        self._check(self.lib.ismc_mlp_sync(self.h))
        return hist


# ----------------------------------------------------------------------------
# surrogate-assisted inverse solve
# ----------------------------------------------------------------------------
def _grid(nmua=48, nmus=48):
    a = np.linspace(LO[0], HI[0], nmua)
    s = np.linspace(LO[1], HI[1], nmus)
    A, S = np.meshgrid(a, s, indexing="ij")
    return np.stack([A.ravel(), S.ravel()], 1)


def surrogate_solve(sur, engine, meas, sigma, g=0.9, d=0.1, n=1.4, gn_steps=8, verify_packets=1_000_000,
                    seed=7, fallback=True, plain_packets=100_000, plain_max_evals=400):
    """Solve many measurements [m x 3] of (R_d, T_d, T_u) with noise sigma (3,).

    Returns dict with x [m x 2] (mu_a, mu_s'), verified MC values, fallback mask,
    and timings of each phase."""
    import torch
    meas = np.asarray(meas, dtype=np.float64)
    sig = np.asarray(sigma, dtype=np.float64)
    m = len(meas)
    T = {}
    t0 = time.perf_counter()
    # (1) grid proposal: surrogate on a 48 x 48 (ln mu_a, ln mu_s') grid, shared by all
    grid = _grid()
    X = np.concatenate([grid, np.tile([g, d, n], (len(grid), 1))], 1)
    out = sur.forward(X).cpu().numpy()[:, :3].astype(np.float64)
    mt = torch.as_tensor(meas, device="cuda")
    ot = torch.as_tensor(out, device="cuda")
    st = torch.as_tensor(sig, device="cuda")
    best = []
    for a in range(0, m, 2048):
        r = (((ot[None, :, :] - mt[a:a + 2048, None, :]) / st) ** 2).sum(-1)
        best.append(r.argmin(1).cpu().numpy())
    x = grid[np.concatenate(best)].copy()
    T["propose_s"] = time.perf_counter() - t0
    # (2) Gauss-Newton on the surrogate (forward differences, damped)
    t1 = time.perf_counter()
    h = 1e-3
    for _ in range(gn_steps):
        pts = np.concatenate([x, x + [h, 0.0], x + [0.0, h]], 0)
        Xp = np.concatenate([pts, np.tile([g, d, n], (len(pts), 1))], 1)
        o = sur.forward(Xp).cpu().numpy()[:, :3].astype(np.float64)
        f0, fa, fs = o[:m], o[m:2 * m], o[2 * m:]
        J = np.stack([(fa - f0) / h, (fs - f0) / h], 2) / sig[None, :, None]     # m x 3 x 2
        rsd = (meas - f0) / sig                                                   # m x 3
        JtJ = np.einsum("mki,mkj->mij", J, J) + 1e-6 * np.eye(2)
        Jtr = np.einsum("mki,mk->mi", J, rsd)
        dx = np.linalg.solve(JtJ, Jtr[..., None])[..., 0]
        dx = np.clip(dx, -1.0, 1.0)
        x = np.clip(x + dx, LO[:2], HI[:2])
    T["gauss_newton_s"] = time.perf_counter() - t1
    # (3) Monte Carlo verification at the answers: one batched launch
    t2 = time.perf_counter()
    sph = bench_spheres()
    insts = [make_instance(sample_stack(math.exp(x[i, 0]), math.exp(x[i, 1]), g, d, n), sph,
                           verify_packets, seed=seed, stream=i) for i in range(m)]
    res = engine.run_batch(insts)
    V = np.array([[r.mean[1], r.mean[3], r.mean[4]] for r in res])
    VS = np.array([[r.se[1], r.se[3], r.se[4]] for r in res])
    T["verify_s"] = time.perf_counter() - t2
    miss = np.any(np.abs(V - meas) > 3 * np.sqrt(sig ** 2 + VS ** 2), axis=1)
    # (4) fallback to the plain path for the misses
    t3 = time.perf_counter()
    xr = np.exp(x)
    if fallback and miss.any():
        idx = np.nonzero(miss)[0]
        reqs = [make_solve(sample_stack(1.0, 10.0, g, d, n), 1, sph, plain_packets,
                           (meas[i, 0], None, meas[i, 1], meas[i, 2]), x0=tuple(xr[i]),
                           seed=seed + 1, max_evals=plain_max_evals) for i in idx]
        outp = engine.solve_batch(reqs)
        for i, o in zip(idx, outp):
            xr[i] = (o.x[0], o.x[1])
    T["fallback_s"] = time.perf_counter() - t3
    T["total_s"] = time.perf_counter() - t0
    return {"x": xr, "verified": V, "verified_se": VS, "fallback": miss, "timing": T}

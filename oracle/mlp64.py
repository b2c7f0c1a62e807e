"""ORACLE (test infrastructure only): FP64 numpy forward/backward of the
surrogate MLP, for checking the tensor-core kernels' outputs and gradients.

Network: x (5 raw inputs) -> map each feature to [-1, 1] -> 256 -> 256 -> 256
-> 6 with SiLU hidden activations.  Outputs: mu (3) and log-variance s (3).
Loss: mean over rows of sum_k 0.5 * ((y_k - mu_k)^2 / v_k + ln v_k),
v_k = exp(s_k) + floor^2 (Gaussian NLL with a variance floor).

With bf16=True the oracle rounds to bfloat16 exactly where the GPU path stores
bfloat16 (weights, normalised inputs, hidden activations, SiLU derivatives,
output gradient, back-propagated gradients), and otherwise computes in FP64,
so the remaining difference is only the FP32 accumulation order.  Each
normalised input f enters the first layer as bf16(f) + bf16(f - bf16(f)), the
two bf16 columns the GPU path stores for it.
"""
import numpy as np

LO = np.array([np.log(0.01), np.log(1.0), 0.6, 0.02, 1.33])
HI = np.array([np.log(10.0), np.log(100.0), 0.95, 0.5, 1.5])
SHAPES = [(256, 5), (256, 256), (256, 256), (6, 256)]


def unflatten(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = [], 0
    for r, c in SHAPES:
        W = p[o:o + r * c].reshape(r, c)
        o += r * c
        b = p[o:o + r]
        o += r
        out.append((W, b))
    assert o == p.size
    return out


def flatten(grads):
    return np.concatenate([np.concatenate([gW.ravel(), gb.ravel()]) for gW, gb in grads])


def bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(params, x, rnd=lambda a: a):
    layers = unflatten(params)
    f = 2.0 * (np.asarray(x, dtype=np.float64) - LO) / (HI - LO) - 1.0
    hi = rnd(f)
    h = hi + rnd(f - hi)
    acts, gates = [h], []
    for W, b in layers[:3]:
        z = h @ rnd(W).T + b
        s = _sig(z)
        h = rnd(z * s)
        acts.append(h)
        gates.append(rnd(s * (1 + z * (1 - s))))
    W, b = layers[3]
    out = h @ rnd(W).T + b
    return out, acts, gates


VAR_FLOOR = 3e-4      # standard-deviation floor of the loss (the GPU kernel's kVarFloor)


def loss_and_grad(params, x, y, bf16_emulation=False, floor=VAR_FLOOR):
    """Gaussian NLL with variance v = exp(s) + floor^2:
    mean over rows of sum_k 0.5 (d^2 / v + ln v), d = y - mu."""
    rnd = bf16 if bf16_emulation else (lambda a: a)
    layers = unflatten(params)
    out, acts, gates = forward(params, x, rnd)
    y = np.asarray(y, dtype=np.float64)
    B = out.shape[0]
    mu, s = out[:, :3], out[:, 3:6]
    d = y - mu
    es = np.exp(s)
    v = es + floor * floor
    loss = np.mean(np.sum(0.5 * (d * d / v + np.log(v)), axis=1))
    dout = np.concatenate([-d / v, 0.5 * (es / v) * (1 - d * d / v)], axis=1) / B
    dout = rnd(dout)
    grads = [None] * 4
    W4, _ = layers[3]
    grads[3] = (dout.T @ acts[3], dout.sum(0))
    dz = rnd((dout @ rnd(W4)) * gates[2])
    for l in (2, 1, 0):
        grads[l] = (dz.T @ acts[l], dz.sum(0))
        if l == 0:
            break
        W, _ = layers[l]
        dz = rnd((dz @ rnd(W)) * gates[l - 1])
    return loss, flatten(grads)

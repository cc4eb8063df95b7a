"""ORACLE -- test infrastructure, not product code.

CPU restatement (numpy) of the surrogate network that
phasefield_coarsening_gb300/csrc/ppf_surrogate.cu and ppf_nn_conv.cu run on
the GPU: features, six 3x3x3 convolutions (periodic halos, or mirrored no-flux
halos for inference) with SiLU, the residual
output, the squared-error loss against a stencil target, and the full
backward pass.  The reference has no learned component; the network stands
in for k_steps calls of its explicit step (phasefield.c:301-403), whose own
restatement is oracle/ppf_oracle.c.

Two modes:
  rounding="device": BF16 rounding at exactly the points where the device
      stores BF16 (features, weights, activations, pre-activations, the
      gradients of pre-activations), FP64 accumulation elsewhere -- the
      device agrees with this up to FP32 accumulation order;
  rounding=None: plain float64 throughout, for finite-difference checks of
      the backward pass itself.

Only tests/ import this module.
"""
from __future__ import annotations

import numpy as np

LAYERS = 6
N_FEATURES = 5          # input channels in use (etaS, etaL, composition, two BF16 residuals)


def bf16(a):
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layer_channels(width):
    ch = [16, width, width, width, width, width, 16]
    return [(ch[i], ch[i + 1]) for i in range(LAYERS)]


def unflatten(params, width):
    """Flat parameter vector -> [(W[27][co][ci], b[co])] per layer (float64)."""
    out, off = [], 0
    for ci, co in layer_channels(width):
        n = 27 * co * ci
        W = np.asarray(params[off:off + n], dtype=np.float64).reshape(27, co, ci)
        off += n
        b = np.asarray(params[off:off + co], dtype=np.float64)
        off += co
        out.append((W, b))
    assert off == len(params)
    return out


def flatten(layers):
    return np.concatenate([np.concatenate([W.ravel(), b]) for W, b in layers])


def init_params(width, seed=0, last_scale=0.0):
    """Seeded uniform initialisation (variance 1/fan_in over the used input
    channels); the output layer is scaled by last_scale (0: the network
    starts as the identity map)."""
    rng = np.random.default_rng(seed)
    layers = []
    for li, (ci, co) in enumerate(layer_channels(width)):
        ci_used = N_FEATURES if li == 0 else ci
        co_used = 3 if li == LAYERS - 1 else co
        a = np.sqrt(3.0 / (27 * ci_used))
        W = np.zeros((27, co, ci))
        W[:, :co_used, :ci_used] = rng.uniform(-a, a, size=(27, co_used, ci_used))
        b = np.zeros(co)
        if li == LAYERS - 1:
            W *= last_scale
        layers.append((W, b))
    return flatten(layers).astype(np.float32)


def taps():
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                yield (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1), dz, dy, dx


def conv(x, W, bc="periodic"):
    """y[co, v] = sum_tap W[tap] @ x[:, v + d(tap)]; x (ci, z, y, x).  Halo:
    periodic images, or for "noflux" the mirror of the reference's no-flux
    fill (ghost -1 = cell 0, ghost n = cell n-1, phasefield.c:1151-1189)."""
    y = np.zeros((W.shape[1],) + x.shape[1:])
    if bc == "periodic":
        for t, dz, dy, dx in taps():
            xs = np.roll(x, shift=(-dz, -dy, -dx), axis=(1, 2, 3))
            y += np.einsum("oc,czyx->ozyx", W[t], xs, optimize=True)
        return y
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1)), mode="edge")
    nz, ny, nx = x.shape[1:]
    for t, dz, dy, dx in taps():
        xs = xp[:, 1 + dz:1 + dz + nz, 1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx]
        y += np.einsum("oc,czyx->ozyx", W[t], xs, optimize=True)
    return y


def conv_adjoint(g, W):
    """x-gradient of conv: dx[ci, u] = sum_tap W[tap]^T g[:, u - d(tap)]."""
    dx_ = np.zeros((W.shape[2],) + g.shape[1:])
    for t, dz, dy, dx in taps():
        gs = np.roll(g, shift=(dz, dy, dx), axis=(1, 2, 3))
        dx_ += np.einsum("oc,ozyx->czyx", W[t], gs, optimize=True)
    return dx_


def conv_wgrad(x, g):
    """dW[tap][co][ci] = sum_v g[co, v] x[ci, v + d(tap)]."""
    out = np.zeros((27, g.shape[0], x.shape[0]))
    for t, dz, dy, dx in taps():
        xs = np.roll(x, shift=(-dz, -dy, -dx), axis=(1, 2, 3))
        out[t] = np.einsum("ozyx,czyx->oc", g, xs, optimize=True)
    return out


def silu(h):
    return h / (1.0 + np.exp(-h))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def features(eS, eL, c, cfg):
    """16-channel input of the first layer, computed in FP32 like the device."""
    eS = np.asarray(eS, np.float32)
    eL = np.asarray(eL, np.float32)
    c = np.asarray(c, np.float32)
    s2, l2 = eS * eS, eL * eL
    h = s2 / np.maximum(s2 + l2, np.float32(1e-30))
    cS, cL, kc = np.float32(cfg["c_solid"]), np.float32(cfg["c_liquid"]), np.float32(cfg["in_scale_c"])
    f2 = (c - (cL + (cS - cL) * h)) * kc
    rS = (eS - bf16(eS).astype(np.float32)) * np.float32(256.0)
    rL = (eL - bf16(eL).astype(np.float32)) * np.float32(256.0)
    f = np.zeros((16,) + eS.shape)
    f[0], f[1], f[2], f[3], f[4] = eS, eL, f2, rS, rL
    return f


def forward(state, params, cfg, rounding="device", bc="periodic"):
    """Network output (3 channels, in units of out_scale) and the tape."""
    r = bf16 if rounding == "device" else (lambda a: np.asarray(a, np.float64))
    layers = unflatten(params, cfg["width"])
    a = r(features(*state, cfg))
    tape = {"a": [a], "z": []}
    for li in range(LAYERS - 1):
        W, b = layers[li]
        h = conv(a, r(W), bc) + b[:, None, None, None]
        tape["z"].append(r(h))
        a = r(silu(h))
        tape["a"].append(a)
    W, b = layers[-1]
    out = conv(a, r(W), bc) + b[:, None, None, None]
    return out[:3], tape


def loss_and_grad(state, target, params, cfg, rounding="device"):
    """Loss of the device's EPI_LOSS epilogue and the gradient of every parameter."""
    r = bf16 if rounding == "device" else (lambda a: np.asarray(a, np.float64))
    layers = unflatten(params, cfg["width"])
    pred, tape = forward(state, params, cfg, rounding)
    n = pred[0].size
    osc = np.asarray(cfg["out_scale"], np.float32)
    lw = np.asarray(cfg["loss_weight"], np.float64) / (3.0 * n)
    s0 = [np.asarray(s, np.float32) for s in state]
    s1 = [np.asarray(s, np.float32) for s in target]
    t = np.stack([((s1[k] - s0[k]) / osc[k]).astype(np.float64) for k in range(3)])
    diff = pred - t
    loss = float(np.sum(lw[:, None, None, None] * diff * diff))
    g = np.zeros((16,) + pred.shape[1:])
    g[:3] = 2.0 * lw[:, None, None, None] * diff
    grads = [None] * LAYERS
    db = g.sum(axis=(1, 2, 3))
    gz = r(g)
    for li in range(LAYERS - 1, -1, -1):
        W, _ = layers[li]
        dW = conv_wgrad(tape["a"][li], gz)
        grads[li] = (dW, db)
        if li == 0:
            break
        da = conv_adjoint(gz, r(W))
        dz = da * dsilu(tape["z"][li - 1])
        db = dz.sum(axis=(1, 2, 3))
        gz = r(dz)
    return loss, flatten(grads)

"""CPU oracle of the step-size / switch MLP (test infrastructure only).

A numpy restatement of the network the GPU kernels run (16 -> 64 -> 64 -> 2,
ReLU, BF16 weights and activations, FP32 accumulation) and of its loss and
backward pass, with BF16 rounding at exactly the points where the kernels
round: normalised features, weights, hidden activations, and the hidden-layer
gradients dZ2 and dZ1. ``exact=True`` drops every rounding and works in
float64, which is what the finite-difference check of the backward pass uses.

The network has no counterpart in the reference (its step-size control is
SciPy's dopri5 / dop853); parity is pinned by the finite-difference check of
this file's gradients and by the kernels' agreement with this file.

Parameter vector (floats): W1T[64][16] b1[64] W2T[64][64] b2[64] W3T[8][64]
b3[8] | xmu[16] xsig[16] ymu[8] ysig[8]. Sample: 16 raw features, the step
target (NaN: none), the switch label (-1: none).
"""
import numpy as np

NTRAIN = 5768
NPARAMS = 5816
SAMPLE = 18

_OFF = {}
_o = 0
for _name, _shape in (("W1T", (64, 16)), ("b1", (64,)), ("W2T", (64, 64)), ("b2", (64,)), ("W3T", (8, 64)),
                      ("b3", (8,)), ("xmu", (16,)), ("xsig", (16,)), ("ymu", (8,)), ("ysig", (8,))):
    _OFF[_name] = (_o, _shape)
    _o += int(np.prod(_shape))
assert _o == NPARAMS


def unpack(p):
    p = np.asarray(p, dtype=np.float32)
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in _OFF.items()}


def pack(d):
    p = np.zeros(NPARAMS, np.float32)
    for k, (o, s) in _OFF.items():
        p[o:o + int(np.prod(s))] = np.asarray(d[k], np.float32).ravel()
    return p


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def _rnd(x, exact):
    return np.asarray(x, np.float64) if exact else bf16(np.asarray(x, np.float32)).astype(np.float64)


def forward(params, feats, exact=False):
    """Outputs in target units, [n][2], plus the intermediate values."""
    d = unpack(params)
    f = np.asarray(feats, np.float32).reshape(-1, 16)
    if exact:
        xn = (f.astype(np.float64) - d["xmu"]) / d["xsig"]
    else:
        xn = ((f - d["xmu"]) / d["xsig"]).astype(np.float32)
    X = _rnd(xn, exact)
    W1, W2, W3 = (_rnd(d[k], exact) for k in ("W1T", "W2T", "W3T"))
    Z1 = X @ W1.T + d["b1"]
    H1 = _rnd(np.maximum(Z1, 0), exact)
    Z2 = H1 @ W2.T + d["b2"]
    H2 = _rnd(np.maximum(Z2, 0), exact)
    O = H2 @ W3[:2].T + d["b3"][:2]
    out = O * d["ysig"][:2] + d["ymu"][:2]
    return out, dict(X=X, H1=H1, H2=H2, O=O, W1=W1, W2=W2, W3=W3)


def loss_and_grad(params, samples, switch_weight=1.0, exact=False):
    """Mean loss (step part, switch part) and its gradient w.r.t. the trainable
    parameters, laid out like the parameter vector's first NTRAIN floats."""
    d = unpack(params)
    s = np.asarray(samples, np.float32).reshape(-1, SAMPLE)
    B = s.shape[0]
    _, v = forward(params, s[:, :16], exact)
    X, H1, H2, O, W2, W3 = v["X"], v["H1"], v["H2"], v["O"], v["W2"], v["W3"]
    tg = s[:, 16].astype(np.float64)
    tn = (np.nan_to_num(tg) - d["ymu"][0]) / d["ysig"][0]
    lab = s[:, 17].astype(np.float64)
    has = lab >= 0
    d0 = np.where(np.isnan(tg), 0.0, O[:, 0] - tn)  # NaN target: switch-labelled sample
    sg = 1.0 / (1.0 + np.exp(-O[:, 1]))
    d1 = np.where(has, switch_weight * (sg - lab), 0.0)
    o1 = O[:, 1]
    l1 = np.where(has, switch_weight * (np.maximum(o1, 0) - o1 * lab + np.log1p(np.exp(-np.abs(o1)))), 0.0)
    loss = (0.5 * np.sum(d0 * d0) / B, np.sum(l1) / B)
    dO = np.stack([d0, d1], 1) / B
    if not exact:
        dO = dO.astype(np.float32).astype(np.float64)
    g = {k: np.zeros(_OFF[k][1]) for k in ("W1T", "b1", "W2T", "b2", "W3T", "b3")}
    g["W3T"][:2] = dO.T @ H2
    g["b3"][:2] = dO.sum(0)
    dZ2 = _rnd((dO @ W3[:2]) * (H2 > 0), exact)
    g["W2T"] = dZ2.T @ H1
    g["b2"] = dZ2.sum(0)
    dZ1 = _rnd((dZ2 @ W2) * (H1 > 0), exact)
    g["W1T"] = dZ1.T @ X
    g["b1"] = dZ1.sum(0)
    grad = np.concatenate([g[k].ravel() for k in ("W1T", "b1", "W2T", "b2", "W3T", "b3")])
    return loss, grad


def finite_difference(params, samples, idx, switch_weight=1.0, eps=1e-4):
    """Central differences of the exact (float64) mean loss at parameter indices idx."""
    p = np.asarray(params, np.float64)
    out = np.zeros(len(idx))

    def total(q):
        # float64 evaluation: pack() would round to float32, so evaluate directly
        return sum(_loss64(q, samples, switch_weight))

    for j, i in enumerate(idx):
        a = p.copy(); a[i] += eps
        b = p.copy(); b[i] -= eps
        out[j] = (total(a) - total(b)) / (2 * eps)
    return out


def _loss64(p, samples, switch_weight):
    d = {k: np.asarray(p[o:o + int(np.prod(s))], np.float64).reshape(s) for k, (o, s) in _OFF.items()}
    s = np.asarray(samples, np.float64).reshape(-1, SAMPLE)
    X = (s[:, :16] - d["xmu"]) / d["xsig"]
    H1 = np.maximum(X @ d["W1T"].T + d["b1"], 0)
    H2 = np.maximum(H1 @ d["W2T"].T + d["b2"], 0)
    O = H2 @ d["W3T"][:2].T + d["b3"][:2]
    tn = (s[:, 16] - d["ymu"][0]) / d["ysig"][0]
    lab = s[:, 17]
    has = lab >= 0
    o1 = O[:, 1]
    l1 = np.where(has, switch_weight * (np.maximum(o1, 0) - o1 * lab + np.log1p(np.exp(-np.abs(o1)))), 0.0)
    l0 = np.where(np.isnan(tn), 0.0, (O[:, 0] - np.nan_to_num(tn)) ** 2)
    return 0.5 * np.mean(l0), np.mean(l1)

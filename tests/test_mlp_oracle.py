"""CPU checks of the MLP oracle: its backward pass against central finite
differences of the float64 loss, and its BF16-rounded variant (what the GPU
kernels compute) against the exact one."""
import numpy as np

from oracle import mlp_oracle as MO
from rapt_gb300 import learned


def _problem(seed=0, n=96):
    rng = np.random.default_rng(seed)
    p = learned.init_params(seed)
    feats = rng.normal(size=(n, 16)).astype(np.float32) * 2 + 1
    feats[:, 14:] = 0
    target = (np.sin(feats[:, 0]) + 0.3 * feats[:, 3]).astype(np.float32)
    lab = np.where(rng.random(n) < 0.5, (feats[:, 1] > 1).astype(np.float32), -1.0).astype(np.float32)
    # a fifth of the samples carry only a switch label (no step target)
    sw_only = rng.random(n) < 0.2
    target[sw_only] = np.nan
    lab[sw_only] = (feats[sw_only, 2] > 0).astype(np.float32)
    samples = np.column_stack([feats, target, lab]).astype(np.float32)
    p = learned.set_normalisation(p, samples)
    # nonzero biases so every parameter block matters
    d = MO.unpack(p)
    d["b1"][:] = rng.normal(size=64) * 0.1
    d["b2"][:] = rng.normal(size=64) * 0.1
    d["b3"][:2] = rng.normal(size=2) * 0.1
    return MO.pack(d), samples


def test_layout_constants_match_native():
    from rapt_gb300 import _native as N
    assert MO.NPARAMS == N.MLP_NPARAMS and MO.NTRAIN == N.MLP_NTRAIN and MO.SAMPLE == N.MLP_SAMPLE


def test_exact_gradient_matches_finite_differences():
    p, s = _problem()
    (l0, l1), g = MO.loss_and_grad(p, s, switch_weight=0.7, exact=True)
    assert l0 > 0 and l1 > 0
    rng = np.random.default_rng(1)
    # a sample of every parameter block: W1T, b1, W2T, b2, W3T rows 0-1, b3[0:2]
    blocks = [(0, 1024), (1024, 1088), (1088, 5184), (5184, 5248), (5248, 5376), (5760, 5762)]
    idx = np.concatenate([rng.choice(np.arange(a, b), size=min(12, b - a), replace=False) for a, b in blocks])
    fd = MO.finite_difference(p, s, idx, switch_weight=0.7, eps=1e-6)
    # ReLU kinks make a few differences one-sided; the bulk must agree tightly
    rel = np.abs(fd - g[idx]) / (np.abs(g[idx]) + 1e-4 * np.abs(g).max())
    assert np.median(rel) < 1e-5 and np.mean(rel < 1e-3) > 0.95, (np.median(rel), rel.max())


def test_unused_output_rows_get_no_gradient():
    p, s = _problem(2)
    _, g = MO.loss_and_grad(p, s)
    assert np.all(g[5248 + 2 * 64:5248 + 8 * 64] == 0) and np.all(g[5760 + 2:5768] == 0)


def test_bf16_gradient_close_to_exact():
    p, s = _problem(3, n=256)
    _, ge = MO.loss_and_grad(p, s, exact=True)
    _, gb = MO.loss_and_grad(p, s, exact=False)
    cos = ge @ gb / np.linalg.norm(ge) / np.linalg.norm(gb)
    assert cos > 0.999, cos
    assert np.linalg.norm(gb - ge) / np.linalg.norm(ge) < 0.05


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0], np.float32)
    r = MO.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0 and r[4] == -2.5 and r[5] == 0

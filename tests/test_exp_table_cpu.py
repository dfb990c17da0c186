"""Accuracy of the table-driven exponential that the Newton residual's FP64 branch uses
(exp_tang in sf_poisson.cu; Tang, ACM TOMS 15(2), 1989), restated here with the same
steps and FP32/FP64 split: within 5e-12 relative of exp over [-700, 700]."""
import numpy as np


def exp_tang(x):
    x = np.asarray(x, np.float64)
    n = np.rint(x * 92.33248261689366).astype(np.int64)
    r = x - n * 0.010830424696249145
    rf = r.astype(np.float32)
    q = rf * (np.float32(0.5) + rf * (np.float32(1 / 6) + rf * np.float32(1 / 24)))
    p = r + r * q.astype(np.float64)
    t = 2.0 ** ((n & 63) / 64.0)
    e = t + t * p
    return np.ldexp(e, (n >> 6).astype(np.int32))


def test_exp_tang_accuracy():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-700, 700, 200000), rng.uniform(-1, 1, 200000),
                        np.arange(-700, 701, dtype=np.float64), (np.arange(-64, 65) * np.log(2) / 64)])
    ref = np.exp(x)
    rel = np.abs(exp_tang(x) - ref) / ref
    assert rel.max() < 5e-12, rel.max()

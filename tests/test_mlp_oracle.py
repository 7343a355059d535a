"""The numpy oracle of the surrogate network (oracle/mlp_oracle.py), pinned before it
judges the GPU kernels: BF16 rounding on known values, the exact backward pass against
finite differences, and the BF16-emulating backward pass close to the exact one."""

import numpy as np


def _params(seed):
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..",
                                    "hoomd-oxdna_gb300"))
    from oxdna import surrogate
    p = surrogate.init_params(seed)[0].astype(np.float64)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    p[1024:1088] = rng.normal(0, 0.1, 64)
    p[5184:5248] = rng.normal(0, 0.1, 64)
    p[9344:9408] = rng.normal(0, 0.1, 64)
    p[9472] = 0.3
    return p


def test_bf16_rounding_known_values():
    from oracle import mlp_oracle as M
    assert M.bf16(np.float32(1.0)) == 1.0
    # 1 + 2^-8 lies halfway between 1 and 1 + 2^-7: ties to even -> 1
    assert M.bf16(np.float32(1.0 + 2.0 ** -8)) == 1.0
    assert M.bf16(np.float32(1.0 + 3 * 2.0 ** -8)) == 1.0 + 2.0 ** -6
    assert M.bf16(np.float32(-3.140625)) == -3.140625
    assert M.bf16(np.float32(1.0 + 2.0 ** -9)) == 1.0


def test_exact_backward_matches_finite_differences():
    from oracle import mlp_oracle as M
    p = _params(0)
    rng = np.random.Generator(np.random.PCG64(5))
    x = rng.normal(size=(24, 7))
    yt = rng.normal(size=24)
    g = M.loss_gradient_exact(p, x, yt)
    idx = np.concatenate([rng.choice(np.arange(0, 1024).reshape(64, 16)[:, :7].ravel(), 6),
                          rng.integers(1024, 9473, 24), [9472]])
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (M.loss_exact(pp, x, yt) - M.loss_exact(pm, x, yt)) / (2 * h)
        assert abs(fd - g[k]) < 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def test_bf16_backward_close_to_exact():
    from oracle import mlp_oracle as M
    p = _params(1)
    rng = np.random.Generator(np.random.PCG64(6))
    x = rng.normal(size=(64, 7))
    yt = rng.normal(size=64)
    g_exact = M.loss_gradient_exact(p, x, yt)
    g_bf16, _ = M.loss_gradient(p, x.astype(np.float32), yt)
    for a, b in ((0, 1024), (1024, 1088), (1088, 5184), (5248, 9344), (9408, 9473)):
        scale = np.abs(g_exact[a:b]).max()
        assert np.abs(g_bf16[a:b] - g_exact[a:b]).max() < 0.05 * scale

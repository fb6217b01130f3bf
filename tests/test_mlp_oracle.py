"""CPU checks of the proposal MLP's FP64 oracle and of the class encoding."""
import numpy as np


def test_oracle_gradient_matches_finite_differences():
    import mlp_oracle as mo

    rng = np.random.default_rng(0)
    n_par = 96 * 128 + 128 + 128 * 128 + 128 + 128 * 160 + 160
    p = rng.normal(0, 0.1, n_par)
    x = rng.normal(0, 1, (7, 96))
    y = rng.integers(0, 160, 7)
    loss, g = mo.loss_grad(p, x, y)
    assert np.isfinite(loss) and g.shape == (n_par,)
    idx = rng.choice(n_par, 60, replace=False)
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp, _ = mo.loss_grad(q, x, y)
        q[i] -= 2 * h
        lm, _ = mo.loss_grad(q, x, y)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_round_trip():
    import mlp_oracle as mo

    x = np.array([0.0, 1.0, -2.5, 3.140625, 1e-3, 65504.0], np.float32)
    b = mo.f32_to_bf16(x)
    back = mo.bf16_to_f64(b)
    assert np.all(np.abs(back - x) <= np.abs(x) * 2.0 ** -8)
    # ties round to even: 1 + 2^-8 lies halfway between 1 and 1 + 2^-7
    assert mo.f32_to_bf16(np.array([1.0 + 2.0 ** -8], np.float32))[0] == 0x3F80


def test_class_encoding_round_trip():
    from ecmgenerator_gb300 import proposal as P

    assert P.decode_class(P.CLS_PREF) == ("pref", -1, -1)
    for q in range(16):
        assert P.decode_class(P.CLS_SINGLE + q) == ("single", q, -1)
        assert P.decode_class(P.CLS_CIRCLE + q) == ("circle", q, -1)
        for lo in range(q):
            assert P.decode_class(P.CLS_PAIR + q * (q - 1) // 2 + lo) == ("pair", q, lo)
    assert P.CLS_PAIR + 16 * 15 // 2 == P.CLS_CIRCLE
    assert P.CLS_CIRCLE + 16 == P.CLS_OTHER
    assert P.decode_class(P.CLS_OTHER)[0] == "other"

"""The CPU oracle of the learned warm-start network (oracle/lws_oracle.py):
its analytic gradient against central finite differences of its own loss in
exact FP64 (bf16=False), along random directions and per layer."""
import numpy as np

from oracle import lws_oracle as lo


def test_lws_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(11)
    H, W = 16, 24
    w = np.concatenate([rng.standard_normal(s.stop - s.start) * (np.sqrt(2.0 / 9) if i in (0, 7)
                                                                   else np.sqrt(2.0 / 288))
                        for i, s in enumerate(lo.layer_slices())])
    x = rng.standard_normal((H, W))
    t = rng.standard_normal((H, W)) * 0.1
    loss, g, _ = lo.loss_grad(w, x, t, bf16=False)
    assert np.isfinite(loss) and g.shape == (lo.NPARAMS,)
    eps = 1e-6
    dirs = [rng.standard_normal(lo.NPARAMS) for _ in range(3)]
    for s in lo.layer_slices():  # one direction confined to each layer
        v = np.zeros(lo.NPARAMS)
        v[s] = rng.standard_normal(s.stop - s.start)
        dirs.append(v)
    for v in dirs:
        lp = lo.loss_grad(w + eps * v, x, t, bf16=False)[0]
        lm = lo.loss_grad(w - eps * v, x, t, bf16=False)[0]
        fd = (lp - lm) / (2 * eps)
        an = float(g @ v)
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-3 * np.linalg.norm(g) * np.linalg.norm(v)), (fd, an)


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 0.0])
    r = lo.bf16_round(v)
    # BF16 keeps 8 significand bits: the spacing at 1 is 2^-7
    assert r[0] == 1.0 and r[4] == -2.5 and r[5] == 0.0
    assert r[1] == 1.0               # 1 + 2^-8: a tie, to the even neighbour 1
    assert r[2] == 1.0               # 1 + 2^-9: below half a spacing
    assert r[3] == 1.0 + 2 ** -7     # 1 + 3 2^-9: above half a spacing

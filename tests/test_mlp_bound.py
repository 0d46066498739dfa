"""oracle.mlp_forward_bound is a sound per-element bound: a float32
restatement of the network that sums each pre-activation's products in a
random order (as a tensor core may), adds the bias in float32 and rounds the
activations to BF16, stays within the bound on every element.  CPU only."""
import numpy as np


def fp32_forward(orc, params, X, rng):
    P = orc.mlp_unpack(params)
    Ws = [orc.bf16(P["W1"]).astype(np.float32), orc.bf16(P["W2"]).astype(np.float32),
          orc.bf16(P["W3"]).astype(np.float32)]
    bs = [P["b1"].astype(np.float32), P["b2"].astype(np.float32), P["b3"].astype(np.float32)]
    H = orc.bf16(X).astype(np.float32)
    for layer in range(3):
        W, b = Ws[layer], bs[layer]
        terms = H[:, None, :] * W[None, :, :]  # exact: BF16 x BF16 fits FP32
        order = rng.permutation(W.shape[1])
        acc = np.zeros(terms.shape[:2], np.float32)
        for k in order:
            acc = (acc + terms[:, :, k]).astype(np.float32)
        Z = (acc + b[None, :]).astype(np.float32)
        if layer == 2:
            break
        H = orc.bf16(np.maximum(Z, np.float32(0))).astype(np.float32)
    return (Z[:, :3] + X[:, 8:11].astype(np.float32)).astype(np.float32)


def test_forward_bound_holds_for_fp32_accumulation_orders(orc):
    rng = np.random.default_rng(5)
    params = np.zeros(6288, np.float32)
    params[:-16] = (rng.normal(size=6288 - 16) * 0.1).astype(np.float32)
    P = orc.mlp_unpack(params)
    P["W3"][3:] = 0
    params = orc.mlp_pack(P)
    X = rng.normal(size=(400, 16)).astype(np.float32)
    Y, bound = orc.mlp_forward_bound(params, X)
    worst = 0.0
    for trial in range(4):
        y = fp32_forward(orc, params, X, rng)
        err = np.abs(y.astype(np.float64) - Y)
        assert np.all(err <= bound), float((err / bound).max())
        worst = max(worst, float((err / bound).max()))
    assert worst > 0.0  # the check is not vacuous: the orders do move the result

"""The GJK warm-start network on the tensor cores (tcgen05) against its
float64 restatement, and what it gains over plain GJK.

Forward outputs and training gradients are compared with
oracle.mlp_forward_backward, which rounds to BF16 where the kernels do;
the remaining differences come from the FP32 accumulation order inside the
tensor cores and the odd BF16 rounding it flips.  Forward outputs are held
element by element to oracle.mlp_forward_bound (the FP32 accumulation error
of K = 16 and 64 products, and the BF16 steps an activation can take within
it, carried through |W|); gradient elements to 2^-6 of their sums of
|terms| (a BF16 step is 2^-8 of a term)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def tiny_engine(sd):
    from stardust_gb300 import scenes
    pts, pos, quat, vel, mass, cfg, dt = scenes.hull_box(8, seed=0, box=(0.2, 0.2, 0.2))
    eng = sd.DEMEngine(cfg)
    sd.add_hull_scene(eng, pts, pos, quat, vel, mass)
    eng.prepare()
    return eng


def random_batch(rng, n):
    X = rng.normal(size=(n, 16)).astype(np.float32)
    X[:, 12:] = 0
    X[:, 7] = rng.random(n) < 0.7
    t = rng.normal(size=(n, 3))
    T = np.concatenate([t / np.linalg.norm(t, axis=1, keepdims=True), (rng.random((n, 1)) < 0.9)], 1).astype(np.float32)
    return X, T


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("n", [1, 128, 1000, 20_000])
def test_mlp_forward_matches_oracle(sdlib, orc, n):
    import torch
    eng = tiny_engine(sdlib)
    rng = np.random.default_rng(n)
    p = eng.mlp_params()
    p[:-16] += rng.normal(size=p.size - 16).astype(np.float32) * 0.05  # W3 starts at zero: perturb all
    P = orc.mlp_unpack(p)
    P["W3"][3:] = 0
    p = orc.mlp_pack(P)
    eng.set_mlp_params(p)
    X, T = random_batch(rng, n)
    y = eng.mlp_forward(torch.from_numpy(X).cuda()).cpu().numpy()
    Y, bound = orc.mlp_forward_bound(p, X)
    Y2, _, _ = orc.mlp_forward_backward(p, X, T)
    assert np.array_equal(Y, Y2)
    err = np.abs(y[:, :3].astype(np.float64) - Y)
    worst = float((err / np.maximum(bound, 1e-30)).max()) if n else 0.0
    print(f"n={n}: max |y - Y| {err.max():.3e}, max error / bound {worst:.3f}, median bound {np.median(bound):.3e}")
    assert np.all(err <= bound), worst
    assert np.all(y[:, 3] == 0)
    eng.close()


def test_mlp_gradients_match_oracle(sdlib, orc):
    import torch
    eng = tiny_engine(sdlib)
    rng = np.random.default_rng(7)
    X, T = random_batch(rng, 3000)
    p = eng.mlp_params()
    p[:-16] += rng.normal(size=p.size - 16).astype(np.float32) * 0.05  # W3 starts at zero: every layer gets a gradient
    P = orc.mlp_unpack(p)
    P["W3"][3:] = 0
    p = orc.mlp_pack(P)
    eng.set_mlp_params(p)
    g = eng.mlp_train(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda(), 0)
    _, _, gr, ga = orc.mlp_forward_backward(p, X, T, with_abs=True)
    G, R, A = orc.mlp_unpack(g), orc.mlp_unpack(gr), orc.mlp_unpack(ga)
    for k in ("W1", "b1", "W2", "b2", "W3", "b3"):
        err = np.abs(G[k] - R[k])
        lim = 2.0 ** -6 * A[k] + 1e-12
        print(f"{k}: max |g - G| / sum|terms| {float((err / (A[k] + 1e-30)).max()):.2e}, relative L2 {rel(G[k], R[k]):.2e}")
        assert np.all(err <= lim), (k, float((err / lim).max()))
    eng.close()


def test_mlp_training_lowers_the_loss(sdlib, orc):
    import torch
    eng = tiny_engine(sdlib)
    rng = np.random.default_rng(3)
    X, T = random_batch(rng, 4096)
    # a learnable target: the previous-direction input turned 90 degrees about z
    r = np.stack([X[:, 9], -X[:, 8], X[:, 10]], 1)
    T[:, :3] = r / np.maximum(np.linalg.norm(r, axis=1, keepdims=True), 1e-6)
    _, l0, _ = orc.mlp_forward_backward(eng.mlp_params(), X, T)
    eng.mlp_train(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda(), 300, 3e-3)
    _, l1, _ = orc.mlp_forward_backward(eng.mlp_params(), X, T)
    assert l1 < 0.2 * l0, (l0, l1)
    eng.close()


def test_learned_seed_gains_over_plain_gjk(sdlib):
    """Plain GJK logs its separating directions for 30 steps; the network is
    trained on them (on the GPU); then a plain and a learned engine step the
    same scene: identical contact sets and bit-identical states, and the
    learned seed needs far fewer support evaluations per pair."""
    import torch
    from stardust_gb300 import _abi, scenes
    pts, pos, quat, vel, mass, cfg, dt = scenes.hull_box(3000, seed=1, box=(0.4, 0.4, 0.4), spacing=0.0195,
                                                          vmax=0.3)
    mk = lambda: sdlib.DEMEngine(cfg)
    plain = mk()
    sdlib.add_hull_scene(plain, pts, pos, quat, vel, mass)
    plain.prepare()
    X, T = [], []
    for _ in range(30):
        plain.step(dt, 1)
        e = plain.hull_entries()
        selfs = np.repeat(np.arange(len(e["off"]) - 1), np.diff(e["off"]))
        m = (e["partners"] > selfs) & (e["status"] == 0) & (e["feat"][:, 7] == 1)
        d = e["dir"][m, :3]
        X.append(e["feat"][m])
        T.append(np.concatenate([d / np.linalg.norm(d, axis=1, keepdims=True), np.ones((m.sum(), 1))], 1))
    X = torch.from_numpy(np.concatenate(X).astype(np.float32)).cuda()
    T = torch.from_numpy(np.concatenate(T).astype(np.float32)).cuda()
    plain.mlp_train(X, T, 400, 2e-3)
    params = plain.mlp_params()
    plain.close()

    engines = {}
    for mode in (_abi.SD_GJK_SEED_PLAIN, _abi.SD_GJK_SEED_LEARNED, _abi.SD_GJK_SEED_PREVIOUS):
        eng = mk()
        sdlib.add_hull_scene(eng, pts, pos, quat, vel, mass)
        eng.prepare()
        eng.set_mlp_params(params)
        eng.set_gjk_seed(mode)
        engines[mode] = eng
    it = {0: 0, 1: 0, 2: 0}
    pairs = {0: 0, 1: 0, 2: 0}
    for step in range(40):
        for mode, eng in engines.items():
            eng.step(dt, 1)
            st = eng.stats()
            if step >= 10:
                it[mode] += st["gjk_iters"]
                pairs[mode] += st["gjk_pairs"]
        ep, el = engines[0].hull_entries(), engines[1].hull_entries()
        assert np.array_equal(ep["status"] == 1, el["status"] == 1)
    a = engines[0].bodies(_abi.SD_BODY_POSITION)
    b = engines[1].bodies(_abi.SD_BODY_POSITION)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert pairs[0] == pairs[1]
    ratio = it[0] / it[1]
    print(f"mean GJK support evaluations per pair: plain {it[0] / pairs[0]:.3f}, learned {it[1] / pairs[1]:.3f} "
          f"(ratio {ratio:.2f}), previous direction without the network {it[2] / pairs[2]:.3f}")
    assert ratio > 2.0
    for eng in engines.values():
        eng.close()


def test_online_learned_seed_beats_its_untrained_baseline(sdlib):
    """The network trained online during the run (every 5 steps, 10 Adam
    steps on the max-margin directions of the pairs whose cached certificate
    failed) against the same engine untrained -- the previous-direction seed
    (its last layer starts at zero) -- and plain GJK, on 16,384 hulls after
    150 steps: identical contacts and states, and fewer support evaluations
    per pair than the untrained network."""
    from stardust_gb300 import _abi, scenes
    pts, pos, quat, vel, mass, cfg, dt = scenes.hull_box(16_384, seed=2, box=(0.6, 0.6, 0.6), spacing=0.0195,
                                                          vmax=0.3)
    engines = {}
    for name, mode in (("plain", _abi.SD_GJK_SEED_PLAIN), ("previous", _abi.SD_GJK_SEED_PREVIOUS),
                       ("online", _abi.SD_GJK_SEED_LEARNED)):
        eng = sdlib.DEMEngine(cfg)
        sdlib.add_hull_scene(eng, pts, pos, quat, vel, mass)
        eng.prepare()
        eng.set_gjk_seed(mode)
        if name == "online":
            eng.set_gjk_training(5, 10, 2e-3)
        eng.step(dt, 150)
        engines[name] = eng
    it = {k: 0 for k in engines}
    pairs = {k: 0 for k in engines}
    for _ in range(30):
        for name, eng in engines.items():
            eng.step(dt, 1)
            st = eng.stats()
            it[name] += st["gjk_iters"]
            pairs[name] += st["gjk_pairs"]
    ref = engines["plain"]
    for name in ("previous", "online"):
        assert pairs[name] == pairs["plain"]
        assert np.array_equal(ref.hull_entries()["status"] == 1, engines[name].hull_entries()["status"] == 1)
        assert np.array_equal(ref.bodies(_abi.SD_BODY_POSITION).view(np.uint32),
                              engines[name].bodies(_abi.SD_BODY_POSITION).view(np.uint32))
    per = {k: it[k] / pairs[k] for k in it}
    print(f"support evaluations per pair: plain {per['plain']:.4f}, previous direction {per['previous']:.4f}, "
          f"online-trained network {per['online']:.4f}")
    assert per["online"] < per["previous"] and per["plain"] / per["online"] > 2.0
    for eng in engines.values():
        eng.close()

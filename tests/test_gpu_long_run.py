"""Long runs on the GPU against the CPU oracle: 1,000 steps of sphere scenes
and 600 steps of a convex-hull scene with learned GJK seeds.

The reference's own driver is a long stepping loop (sandbox/testDEM.cpp:
118-128, repeated DEMEngine::update).  Here every run is compared bit for
bit with the FP32 oracle at its last step, so ensemble quantities agree
exactly with it; the FP32-vs-FP64 error is stated by running the oracle's
FP64 twin (oracle.run_f64) from the same input, and the ensemble quantities
-- kinetic energy, packing fraction and contact count (oracle.ensemble) --
are asserted within 1 % of the twin.

The 4,096-sphere box holds ~10 contacts at any time, each lasting ~20
steps, so its contact count is a small-number statistic: one grazing
collision that happens in FP32 and not in FP64 (the trajectories diverge,
max |v32 - v64| reaches 0.1 m/s at step 1,000) moves the instantaneous
count by 7 %.  Its ensemble is therefore eight seeded boxes, and the
contact count the mean over all states of all eight runs.  The dense case
(20,000 spheres with radii inflated by 1.2, ~53,000 contacts) is compared
state by state."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def gpu_run(sdlib, pos, vel, cfg, dt, steps):
    """Steps one at a time, recording the contact pairs of states
    1..steps; returns the final state (id order) and the counts."""
    eng = sdlib.DEMEngine(cfg)
    eng.add_spheres(pos, vel)
    eng.prepare()
    counts = [eng.stats()["contacts"]]
    for _ in range(steps):
        eng.step(dt, 1)
        counts.append(eng.stats()["contacts"])
    eng.sync()
    st = eng.stats()
    assert st["device_errors"] == 0 and st["steps"] == steps
    out = (eng.positions(), eng.velocities(), eng.omegas(), np.array(counts[:-1], np.int64), eng.params())
    eng.close()
    return out


def compare(orc, cfg, pos, vel, dt, steps, gp, gv, gw, ep):
    """Bit-exact against the FP32 oracle; returns the FP64 twin's run."""
    n = len(pos)
    p = orc.params_checked(cfg, pos[:, 3], dt, ep)
    op, ov, ow = orc.run(p, pos, vel, orc.with_ids(np.zeros_like(pos), np.arange(n)), steps)
    assert np.array_equal(bits(gp), bits(orc.unsort(op, ow)))
    assert np.array_equal(bits(gv), bits(orc.unsort(ov, ow)))
    assert np.array_equal(bits(gw)[:, :3], bits(orc.unsort(ow, ow))[:, :3])
    return orc.run_f64(p, pos, vel, np.zeros_like(pos), steps)


def within(a, b, tol=0.01):
    return abs(a - b) <= tol * abs(b)


def test_box_lattice_1000_steps_ensemble(sdlib, orc):
    """The 4,096-sphere box (16^3 jittered lattice, r 0.01 m, dt 1e-5 s),
    eight seeds, 1,000 steps each."""
    from stardust_gb300 import scenes
    steps = 1000
    e32, e64, c32, c64 = [], [], [], []
    for seed in range(8):
        pos, vel, cfg, dt = scenes.box_lattice(n_side=16, seed=seed)
        gp, gv, gw, counts, ep = gpu_run(sdlib, pos, vel, cfg, dt, steps)
        dp, dv, dw, counts64 = compare(orc, cfg, pos, vel, dt, steps, gp, gv, gw, ep)
        e32.append(orc.ensemble(gp, gv, gw))
        e64.append(orc.ensemble(dp, dv, dw))
        c32.append(counts)
        c64.append(counts64)
        err = np.abs(gp[:, :3].astype(np.float64) - dp[:, :3]).max()
        print(f"seed {seed}: max |x32 - x64| {err:.3e} m, max |v32 - v64| "
              f"{np.abs(gv[:, :3].astype(np.float64) - dv[:, :3]).max():.3e} m/s, contacts at step {steps}: "
              f"{e32[-1]['contacts']} (FP64 {e64[-1]['contacts']})")
    ke32, ke64 = np.mean([e["kinetic_energy"] for e in e32]), np.mean([e["kinetic_energy"] for e in e64])
    phi32, phi64 = np.mean([e["packing_fraction"] for e in e32]), np.mean([e["packing_fraction"] for e in e64])
    cc32, cc64 = np.mean(np.concatenate(c32)), np.mean(np.concatenate(c64))
    print(f"ensemble of 8: kinetic energy {ke32:.6e} J (FP64 {ke64:.6e}), packing fraction {phi32:.6f} "
          f"(FP64 {phi64:.6f}), contacts per state {cc32:.4f} (FP64 {cc64:.4f})")
    assert within(ke32, ke64) and within(phi32, phi64) and within(cc32, cc64)


def test_dense_pack_1000_steps_ensemble(sdlib, orc):
    """20,000 polydisperse spheres of the settling box with radii inflated by
    1.2 (a dense, overlapping contact network), 1,000 steps at dt 5e-6 s."""
    from stardust_gb300 import scenes
    n, steps = 20_000, 1000
    pos, vel, cfg, dt, phi = scenes.settling_rsa(n, box=scenes.scaled_box(n), seed=2)
    pos = pos.copy()
    pos[:, 3] *= np.float32(1.2)
    cfg.cell = float(2 * pos[:, 3].max())
    gp, gv, gw, counts, ep = gpu_run(sdlib, pos, vel, cfg, dt, steps)
    dp, dv, dw, counts64 = compare(orc, cfg, pos, vel, dt, steps, gp, gv, gw, ep)
    a, b = orc.ensemble(gp, gv, gw), orc.ensemble(dp, dv, dw)
    print(f"FP32 {a}, FP64 {b}; mean contacts over the last 100 states {counts[-100:].mean():.2f} "
          f"(FP64 {counts64[-100:].mean():.2f}); max |x32 - x64| "
          f"{np.abs(gp[:, :3].astype(np.float64) - dp[:, :3]).max():.3e} m")
    assert a["contacts"] > 40_000
    for k in ("kinetic_energy", "packing_fraction", "contacts"):
        assert within(a[k], b[k]), k
    assert within(counts[-100:].mean(), counts64[-100:].mean())


def test_hull_600_steps_with_learned_seeds(sdlib, orc):
    """3,000 convex hulls: the warm-start network is trained on the GPU on
    the separating directions plain GJK logs in the first 20 steps, then
    the scene runs 600 steps with learned seeds beside a plain-GJK engine.
    Seeds change only the iteration count, so both states equal the
    plain-GJK oracle's bit for bit after 600 steps (the oracle starts from
    the engine's initial bodies and principal-frame shapes), and the
    learned run needs fewer support evaluations per pair than plain GJK
    over the whole run."""
    import torch
    from stardust_gb300 import _abi, scenes
    pts, pos, quat, vel, mass, cfg, dt = scenes.hull_box(3000, seed=1, box=(0.4, 0.4, 0.4), spacing=0.0195,
                                                          vmax=0.3)
    warm, steps = 20, 600

    def engine(mode, params=None):
        e = sdlib.DEMEngine(cfg)
        sdlib.add_hull_scene(e, pts, pos, quat, vel, mass)
        e.prepare()
        if params is not None:
            e.set_mlp_params(params)
        e.set_gjk_seed(mode)
        return e

    plain = engine(_abi.SD_GJK_SEED_PLAIN)
    X, T = [], []
    for _ in range(warm):
        plain.step(dt, 1)
        e = plain.hull_entries()
        selfs = np.repeat(np.arange(len(e["off"]) - 1), np.diff(e["off"]))
        m = (e["partners"] > selfs) & (e["status"] == 0) & (e["feat"][:, 7] == 1)
        d = e["dir"][m, :3]
        X.append(e["feat"][m])
        T.append(np.concatenate([d / np.linalg.norm(d, axis=1, keepdims=True), np.ones((m.sum(), 1))], 1))
    plain.mlp_train(torch.from_numpy(np.concatenate(X).astype(np.float32)).cuda(),
                    torch.from_numpy(np.concatenate(T).astype(np.float32)).cuda(), 300, 2e-3)
    params = plain.mlp_params()
    plain.close()

    learned = engine(_abi.SD_GJK_SEED_LEARNED, params)
    plain = engine(_abi.SD_GJK_SEED_PLAIN)
    vs, vc, verts = learned.hull_shapes()
    b = {k: learned.bodies(f) for k, f in (("pos", _abi.SD_BODY_POSITION), ("vel", _abi.SD_BODY_VELOCITY),
                                             ("quat", _abi.SD_BODY_QUATERNION), ("omg", _abi.SD_BODY_OMEGA),
                                             ("ang", _abi.SD_BODY_ANGMOM), ("iinv", _abi.SD_BODY_HULL_INV_INERTIA))}
    H = orc.Hulls(b["pos"], b["vel"], b["quat"], b["omg"], b["ang"], b["iinv"], vs, vc, verts)
    it = {"plain": 0, "learned": 0}
    pairs = {"plain": 0, "learned": 0}
    for _ in range(steps):
        for name, eng in (("plain", plain), ("learned", learned)):
            eng.step(dt, 1)
            st = eng.stats()
            it[name] += st["gjk_iters"]
            pairs[name] += st["gjk_pairs"]
    learned.sync()
    assert learned.stats()["device_errors"] == 0
    p = orc.hull_params(cfg.box_lo, cfg.box_hi, cfg.kn, orc.damp_from(cfg.kn, cfg.restitution), cfg.mu, cfg.gravity,
                        dt, cfg.walls)
    for _ in range(steps):
        out = H.step(p)
    for k, f in (("pos", _abi.SD_BODY_POSITION), ("vel", _abi.SD_BODY_VELOCITY), ("quat", _abi.SD_BODY_QUATERNION),
                 ("omg", _abi.SD_BODY_OMEGA), ("ang", _abi.SD_BODY_ANGMOM)):
        assert np.array_equal(bits(learned.bodies(f)), bits(getattr(H, k))), k
        assert np.array_equal(bits(plain.bodies(f)), bits(getattr(H, k))), k
    e = learned.hull_entries()
    assert np.array_equal(e["off"], out["off"]) and np.array_equal(e["partners"], out["partners"])
    # the same contact set; a seeded run may certify as separated a pair that
    # plain GJK ends as touching (a repeated support point): no force either way
    assert np.array_equal(e["status"] == 1, out["status"] == 1)
    assert np.array_equal(plain.hull_entries()["status"], out["status"])
    assert int((out["status"] == 1).sum()) > 20
    assert pairs["plain"] == pairs["learned"]
    ratio = it["plain"] / it["learned"]
    print(f"{steps} steps: support evaluations per pair plain {it['plain'] / pairs['plain']:.3f}, learned "
          f"{it['learned'] / pairs['learned']:.3f} (ratio {ratio:.2f})")
    assert ratio > 1.5
    learned.close()
    plain.close()

"""Adjoint rollouts (torch.autograd.Function over the GPU step) against central finite
differences of the oracle's rollout (the CPU restatement of the reference step).

Loss: sum of squared distances of the bodies' translations after the rollout to seeded
targets. Newton runs to a tight tolerance so that the finite differences resolve the
converged map. The adjoint differentiates every friction term through its multiplier and
tangent frame (ground, point-triangle and edge-edge), so the check covers friction
between bodies as well as against the ground."""
import dataclasses

import numpy as np
import pytest

from adb_gb300 import scene as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def O(gpu_lib, oracle_lib):
    return oracle_lib


def setup(mu, contact_friction=True):
    sc = S.diff_grid(seed=1, n=2, spacing=1.05, lift=0.56)
    cfg = dataclasses.replace(S.workload_config("diff"), mu=mu, tol=1e-12, pt_friction=contact_friction,
                              ee_friction=contact_friction, max_iter_frame=0)
    rng = np.random.default_rng(7)
    target = sc.q0[:, :3] + rng.uniform(-0.3, 0.3, (sc.n_bodies, 3))
    v0 = np.zeros_like(sc.q0)
    v0[:, :3] = rng.normal(0.0, 0.5, (sc.n_bodies, 3))
    v0[:, 1] -= 1.0
    return sc, cfg, target, v0


def oracle_loss(O, sc, cfg, q0, v0, mu, target, n):
    o = O.OracleSim(sc, dataclasses.replace(cfg, mu=mu))
    o.set_state(q0, v0)
    o.step(n)
    q, _ = o.state()
    return float(((q[:, :3] - target) ** 2).sum())


@pytest.mark.parametrize("mu,contact_friction,bound", [(0.0, True, 1e-5), (0.3, False, 1e-5), (0.3, True, 1e-5)])
def test_adjoint_matches_oracle_finite_differences(O, mu, contact_friction, bound):
    from adb_gb300.abd import ABD
    from adb_gb300.adjoint import rollout
    sc, cfg, target, v0 = setup(mu, contact_friction)
    n = 12
    sim = ABD(sc, cfg)
    q0t = torch.tensor(sc.q0, dtype=torch.float64, requires_grad=True)
    v0t = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
    mut = torch.tensor(mu, dtype=torch.float64, requires_grad=True)
    qT, _ = rollout(sim, q0t, v0t, mut, n, every=4)
    loss = ((qT[:, :3] - torch.tensor(target)) ** 2).sum()
    loss.backward()
    L0 = oracle_loss(O, sc, cfg, sc.q0, v0, mu, target, n)
    assert abs(float(loss.detach()) - L0) <= 1e-8 * abs(L0)
    rng = np.random.default_rng(3)
    h = 1e-5
    pairs = []
    for k in range(3):
        d = rng.normal(size=v0.shape)
        d[:, 3:] = 0.0
        d /= np.linalg.norm(d)
        fd = (oracle_loss(O, sc, cfg, sc.q0, v0 + h * d, mu, target, n) -
              oracle_loss(O, sc, cfg, sc.q0, v0 - h * d, mu, target, n)) / (2 * h)
        ad = float((v0t.grad.numpy() * d).sum())
        print("adjoint v0 direction %d: %.10g fd %.10g" % (k, ad, fd))
        pairs.append((ad, fd))
    # errors relative to the largest directional derivative (the finite differences of a
    # converged Newton solve resolve derivatives to a fraction of the gradient's size)
    scale = max(abs(fd) for _, fd in pairs)
    for k, (ad, fd) in enumerate(pairs):
        assert abs(ad - fd) <= bound * scale, (k, ad, fd, scale)
    if mu > 0:
        fd = (oracle_loss(O, sc, cfg, sc.q0, v0, mu + h, target, n) -
              oracle_loss(O, sc, cfg, sc.q0, v0, mu - h, target, n)) / (2 * h)
        print("adjoint mu: %.10g fd %.10g" % (float(mut.grad), fd))
        assert abs(float(mut.grad) - fd) <= bound * abs(fd), (float(mut.grad), fd)


def test_interleaved_rollouts_keep_their_own_friction(gpu_lib):
    """Two rollouts of one simulation with different mu, then backward on their summed
    loss: each backward pass recomputes its frames (checkpoints every 4) with its own mu,
    so the gradients equal those of each rollout differentiated alone, and the simulation
    is handed back with the state and friction it had."""
    from adb_gb300.abd import ABD
    from adb_gb300.adjoint import rollout
    sc, cfg, target, v0 = setup(0.2, contact_friction=False)
    n = 8
    tgt = torch.tensor(target)

    def grads(mus, together):
        sim = ABD(sc, cfg)
        out = []
        losses = []
        for mu in mus:
            v0t = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
            mut = torch.tensor(mu, dtype=torch.float64, requires_grad=True)
            qT, _ = rollout(sim, torch.tensor(sc.q0), v0t, mut, n, every=4)
            loss = ((qT[:, :3] - tgt) ** 2).sum()
            if together:
                losses.append(loss)
            else:
                loss.backward()
            out.append((v0t, mut))
        if together:
            before = sim.state(), sim.friction
            sum(losses).backward()
            after = sim.state(), sim.friction
            assert after[1] == before[1]
            assert np.array_equal(after[0][0], before[0][0]) and np.array_equal(after[0][1], before[0][1])
        sim.close()
        return [(v.grad.numpy().copy(), float(m.grad)) for v, m in out]

    alone = grads([0.0, 0.3], together=False)
    both = grads([0.0, 0.3], together=True)
    for (ga, ma), (gb, mb) in zip(alone, both):
        assert np.array_equal(ga, gb) and ma == mb


def test_adjoint_state_and_affine_velocity_directions(O):
    """Directions in every component of the initial velocities (translation and affine
    blocks) and of the initial state q0 (translations and affine entries), with contact
    friction between bodies (mu 0.3), against central differences of the oracle."""
    from adb_gb300.abd import ABD
    from adb_gb300.adjoint import rollout
    mu = 0.3
    sc, cfg, target, v0 = setup(mu, True)
    n = 12
    sim = ABD(sc, cfg)
    q0t = torch.tensor(sc.q0, dtype=torch.float64, requires_grad=True)
    v0t = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
    qT, _ = rollout(sim, q0t, v0t, torch.tensor(mu, dtype=torch.float64), n, every=4)
    loss = ((qT[:, :3] - torch.tensor(target)) ** 2).sum()
    loss.backward()
    rng = np.random.default_rng(9)
    h = 1e-5
    pairs = []
    for which in ("v0", "v0", "q0", "q0"):
        d = rng.normal(size=v0.shape)
        if which == "q0":
            d[:, 3:] *= 0.1   # affine entries: a small shear / scale next to the translations
        d /= np.linalg.norm(d)
        if which == "v0":
            fd = (oracle_loss(O, sc, cfg, sc.q0, v0 + h * d, mu, target, n) -
                  oracle_loss(O, sc, cfg, sc.q0, v0 - h * d, mu, target, n)) / (2 * h)
            ad = float((v0t.grad.numpy() * d).sum())
        else:
            fd = (oracle_loss(O, sc, cfg, sc.q0 + h * d, v0, mu, target, n) -
                  oracle_loss(O, sc, cfg, sc.q0 - h * d, v0, mu, target, n)) / (2 * h)
            ad = float((q0t.grad.numpy() * d).sum())
        print("adjoint %s direction: %.10g fd %.10g" % (which, ad, fd))
        pairs.append((which, ad, fd))
    for which in ("v0", "q0"):
        sel = [(ad, fd) for w, ad, fd in pairs if w == which]
        scale = max(abs(fd) for _, fd in sel)
        for ad, fd in sel:
            assert abs(ad - fd) <= 1e-5 * scale, (which, ad, fd, scale)


def test_full_size_rollout_checkpointing():
    """The differentiable-rollout workload at full size: 64 subdivision-2 icospheres,
    mu 0.3, 100 steps; gradients of the seeded-target loss with respect to the 64 x 12
    initial affine velocities and mu. Checkpointing every 10 frames (the backward pass
    recomputes the frames between checkpoints) must give the gradients of keeping every
    frame bit for bit, and the simulation must come back with its state and friction."""
    from adb_gb300.abd import ABD
    from adb_gb300.adjoint import rollout
    sc = S.diff_grid(seed=0)
    cfg = S.workload_config("diff")
    tgt = torch.tensor(S.diff_targets(sc.n_bodies, seed=0))
    out = []
    for every in (1, 10):
        sim = ABD(sc, cfg)
        v0t = torch.zeros(sc.q0.shape, dtype=torch.float64, requires_grad=True)
        mut = torch.tensor(cfg.mu, dtype=torch.float64, requires_grad=True)
        qT, _ = rollout(sim, torch.tensor(sc.q0), v0t, mut, 100, every=every)
        loss = ((qT[:, :3] - tgt) ** 2).sum()
        before = sim.state()
        loss.backward()
        after = sim.state()
        assert np.array_equal(before[0], after[0]) and sim.friction == cfg.mu
        assert np.isfinite(v0t.grad.numpy()).all() and np.isfinite(float(mut.grad))
        out.append((float(loss.detach()), v0t.grad.numpy().copy(), float(mut.grad)))
        sim.close()
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1]) and out[0][2] == out[1][2]
    assert np.abs(out[0][1]).max() > 0.0


def test_full_size_gradients_match_oracle_fd_before_impacts(O):
    """The differentiable-rollout workload at full size (64 subdivision-2 icospheres, mu 0.3,
    the seeded-target loss, gradients with respect to all 64 x 12 initial velocities and
    mu, checkpoints every 10 frames) over its first 20 frames, which carry the ground
    contacts and their friction. Later frames reach impacts where the reference's Newton
    loop does not converge, so finite differences are taken over this horizon. 20 random
    directions, central differences of the oracle with h = 1e-6, Newton tol 1e-12."""
    from adb_gb300.abd import ABD
    from adb_gb300.adjoint import rollout
    sc = S.diff_grid(seed=0)
    cfg = dataclasses.replace(S.workload_config("diff"), tol=1e-12, max_iter_frame=0)
    target = S.diff_targets(sc.n_bodies, seed=0)
    n = 20
    v0 = np.zeros_like(sc.q0)
    sim = ABD(sc, cfg)
    v0t = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
    mut = torch.tensor(cfg.mu, dtype=torch.float64, requires_grad=True)
    qT, _ = rollout(sim, torch.tensor(sc.q0), v0t, mut, n, every=10)
    loss = ((qT[:, :3] - torch.tensor(target)) ** 2).sum()
    loss.backward()
    L0 = oracle_loss(O, sc, cfg, sc.q0, v0, cfg.mu, target, n)
    assert abs(float(loss.detach()) - L0) <= 1e-8 * abs(L0)
    rng = np.random.default_rng(20)
    h = 1e-6
    pairs = []
    for _ in range(20):
        d = rng.normal(size=v0.shape)
        d /= np.linalg.norm(d)
        fd = (oracle_loss(O, sc, cfg, sc.q0, v0 + h * d, cfg.mu, target, n) -
              oracle_loss(O, sc, cfg, sc.q0, v0 - h * d, cfg.mu, target, n)) / (2 * h)
        pairs.append((float((v0t.grad.numpy() * d).sum()), fd))
    scale = max(abs(fd) for _, fd in pairs)
    worst = max(abs(ad - fd) for ad, fd in pairs) / scale
    print("full-size directions: worst |ad - fd| / max|fd| = %.2e (max|fd| %.4g)" % (worst, scale))
    assert worst <= 1e-5
    # dL/dmu is small over this horizon (ground friction only, ~4e-4): at h = 1e-6 the
    # central difference resolves it only to its rounding floor (~4 eps |L| / h), so it is
    # checked there against that floor, and at h = 1e-4 (truncation O(h^2), negligible)
    # to 1e-5 relative
    ad = float(mut.grad)
    for hm, bound in ((1e-6, 4 * 2.2e-16 * abs(L0) / 1e-6), (1e-4, 1e-5)):
        fdm = (oracle_loss(O, sc, cfg, sc.q0, v0, cfg.mu + hm, target, n) -
               oracle_loss(O, sc, cfg, sc.q0, v0, cfg.mu - hm, target, n)) / (2 * hm)
        print("full-size dL/dmu: %.10g fd(h=%g) %.10g" % (ad, hm, fdm))
        tol = bound if hm == 1e-6 else bound * abs(fdm)
        assert abs(ad - fdm) <= tol, (hm, ad, fdm, tol)

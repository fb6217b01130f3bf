"""Learned active-set proposal: the MLP kernels against the FP64 oracle, the
trace (features and LP classes), the exact check of proposals, and what the
trained network gains over the method without it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _bf16_rows(torch, n, seed, scale=1.0):
    g = torch.Generator().manual_seed(seed)
    x = (torch.randn(n, 96, generator=g) * scale)
    x[:, 82:] = 0.0
    return x.to(torch.bfloat16).cuda().contiguous()


def _c1_sim(n_agents=1000, seed=7, k=10):
    from ecmgenerator_gb300 import agents as ag
    from ecmgenerator_gb300.simulator import Planner, Simulator

    cfg = ag.scaled("c1", agents=n_agents)
    scene = ag.build_scene(cfg, seed)
    st = ag.spawn_agents(cfg, scene, seed)
    paths = Planner(scene).find_paths(st.pos, st.goal, st.clear)
    paths = [p if p is not None else np.stack([st.pos[i], st.goal[i]]) for i, p in enumerate(paths)]
    sim = Simulator(scene, st.n_slots, 1.0 / 60.0, max_neighbors=k, **ORCA)
    sim.add_agents(st.pos, st.clear, st.pref_speed, paths)
    return sim


def test_mlp_loss_grad_matches_fp64_oracle(lib):
    """the tensor-core forward/backward (BF16 operands, FP32 accumulation)
    against the FP64 oracle that rounds the same operands to BF16: the rest
    is accumulation order and the FP32 elementwise steps"""
    torch = _torch()
    import mlp_oracle as mo
    from ecmgenerator_gb300.proposal import ProposalModel

    m = ProposalModel(seed=3)
    for rows in (512, 3001):  # one M tile per CTA / a ragged batch with split-K weight gradients
        x = _bf16_rows(torch, rows, 11)
        y = torch.randint(0, 160, (rows,), generator=torch.Generator().manual_seed(2)).to(torch.uint8).cuda()
        loss, g = m.loss_grad(x, y)
        p = m.get_params()
        xb = mo.bf16_to_f64(x.view(torch.int16).cpu().numpy().view(np.uint16))
        rl, rg = mo.loss_grad(p, xb, y.cpu().numpy(), bf16_operands=True)
        _, rg64 = mo.loss_grad(p, xb, y.cpu().numpy())
        assert abs(loss - rl) <= 1e-5 * max(1.0, abs(rl))
        err = np.linalg.norm(g - rg) / np.linalg.norm(rg)
        assert err < 5e-4, err
        # the BF16 operands themselves move the gradient by far more than that
        assert np.linalg.norm(g - rg64) / np.linalg.norm(rg64) > 5 * err
        # per block, so that no layer hides behind another
        o = 0
        for name, shp in [("W1", (96, 128)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)),
                          ("W3", (128, 160)), ("b3", (160,))]:
            n = int(np.prod(shp))
            e = np.linalg.norm(g[o:o + n] - rg[o:o + n]) / max(np.linalg.norm(rg[o:o + n]), 1e-30)
            assert e < 5e-4, (rows, name, e)
            o += n
    m.close()


def test_mlp_predict_tensor_cores_matches_bf16_oracle(lib):
    torch = _torch()
    import mlp_oracle as mo
    from ecmgenerator_gb300.proposal import ProposalModel

    m = ProposalModel(seed=5)
    x = _bf16_rows(torch, 4099, 12)  # not a multiple of the 16-row tile
    cls = m.predict(x).cpu().numpy()
    p = m.get_params()
    # oracle with the inference kernel's roundings: BF16 weights and BF16
    # activations between layers, FP32 biases, wide accumulation
    W1, b1, W2, b2, W3, b3 = mo.split(p)
    r = lambda a: mo.bf16_to_f64(mo.f32_to_bf16(a.astype(np.float32)))  # noqa: E731
    xb = mo.bf16_to_f64(x.view(torch.int16).cpu().numpy().view(np.uint16))
    h1 = r(mo.gelu(xb @ r(W1) + b1))
    h2 = r(mo.gelu(h1 @ r(W2) + b2))
    z = h2 @ r(W3) + b3
    ref = z.argmax(1)
    agree = (cls == ref).mean()
    assert agree > 0.995, agree
    bad = np.nonzero(cls != ref)[0]
    gap = z[bad, ref[bad]] - z[bad, cls[bad]]
    assert np.all(gap < 1e-2 * np.abs(z[bad]).max(axis=1) + 1e-3), gap
    m.close()


def test_mlp_predict_pipelined_tiles_match_single_tiles(lib):
    """many tiles per CTA (every pipeline, tiles that wait for their
    features) give the classes that launches of a few tiles give"""
    torch = _torch()
    from ecmgenerator_gb300.proposal import ProposalModel

    m = ProposalModel(seed=6)
    n = 152 * 2 * 4 * 128 + 77
    x = _bf16_rows(torch, n, 13)
    full = m.predict(x).cpu()
    parts = torch.cat([m.predict(x[i:i + 4096].contiguous()).cpu() for i in range(0, n, 4096)])
    assert torch.equal(full, parts)
    m.close()


def test_inference_wait_bound_reports_a_timeout_and_recovers(lib):
    """the inference kernel's bounded mbarrier waits: with a limit of one
    poll the first wait (a feature-tile copy) runs out; the kernel waits for
    its copies, frees its tensor memory and returns, the call reports
    ECMG_ERR_BOUND, and the next call with the default limit gives the
    normal classes"""
    torch = _torch()
    from ecmgenerator_gb300._lib import EcmgError
    from ecmgenerator_gb300.proposal import ProposalModel

    m = ProposalModel(seed=7)
    x = _bf16_rows(torch, 70000, 14)
    want = m.predict(x).cpu()
    assert lib.ecmg_mlp_set_wait_limit(m.h, 1) == 0
    with pytest.raises(EcmgError) as e:
        m.predict(x)
    assert e.value.status == 3  # ECMG_ERR_BOUND
    assert lib.ecmg_mlp_set_wait_limit(m.h, 0) == 0
    assert torch.equal(m.predict(x).cpu(), want)
    assert lib.ecmg_mlp_set_wait_limit(m.h, -1) == 1
    m.close()


def test_mlp_training_learns_a_separable_task(lib):
    torch = _torch()
    from ecmgenerator_gb300.proposal import ProposalModel

    g = torch.Generator().manual_seed(4)
    n = 60000
    x = torch.randn(n, 96, generator=g)
    x[:, 82:] = 0.0
    Wt = torch.randn(96, 8, generator=g)
    y = (x @ Wt).argmax(1).to(torch.uint8)
    xd, yd = x.to(torch.bfloat16).cuda().contiguous(), y.cuda().contiguous()
    m = ProposalModel(seed=1)
    l0, _ = m.loss_grad(xd[:4096], yd[:4096])
    loss, acc = m.train(xd, yd, steps=400, batch=2048, lr=1e-3, seed=9)
    assert np.all(np.isfinite(loss))
    assert loss[-20:].mean() < 0.3 * l0, (l0, loss[-20:].mean())
    pred = m.predict(xd[:8192]).cpu()
    assert (pred == y[:8192]).float().mean().item() > 0.85
    m.close()


def test_trace_features_match_tick_start_state(lib):
    torch = _torch()
    import mlp_oracle as mo

    sim = _c1_sim()
    sim.update(ticks=20)
    pos0 = sim.get_position_data().copy()
    vel0 = sim.get_velocity_data().copy()
    clr = sim.get_clearance_data().copy()
    spd = sim.get_speed_data().copy()
    sim.set_record(True)
    sim.set_trace(True)
    sim.update()
    x, y, slots = sim.get_trace()
    rec = sim.get_record()
    pv = sim.get_preferred_velocity_data()
    active = sim.get_active_flags()
    assert x.shape[0] == len(slots) and len(slots) > 900
    inv_r = np.float32(1.0) / np.float32(5.0)
    checked = 0
    for row, s in enumerate(slots):
        if not active[s]:
            assert np.all(x[row] == 0) and y[row] == 153
            continue
        f = np.zeros(96, np.float32)
        nb = rec["nbr_ids"][s][:rec["nbr_count"][s]][:16]
        for q, j in enumerate(nb):
            f[5 * q + 0] = (pos0[j, 0] - pos0[s, 0]) * inv_r
            f[5 * q + 1] = (pos0[j, 1] - pos0[s, 1]) * inv_r
            f[5 * q + 2] = (vel0[s, 0] - vel0[j, 0]) * np.float32(0.5)
            f[5 * q + 3] = (vel0[s, 1] - vel0[j, 1]) * np.float32(0.5)
            f[5 * q + 4] = clr[j] + clr[s]
        im = np.float32(1.0) / spd[s]
        f[80] = pv[s, 0] * im
        f[81] = pv[s, 1] * im
        assert np.array_equal(x[row], mo.f32_to_bf16(f)), (row, s)
        checked += 1
    assert checked > 900
    sim.close()


def _pair(n_agents=1000, ticks=30, mode=None):
    """two simulators in the same state (the tick is deterministic)"""
    from ecmgenerator_gb300.simulator import set_lp_mode

    a, b = _c1_sim(n_agents), _c1_sim(n_agents)
    if mode:
        set_lp_mode(b, mode, 2)
    a.update(ticks=ticks)
    b.update(ticks=ticks)
    assert np.array_equal(a.get_position_data(), b.get_position_data())
    return a, b


@pytest.mark.parametrize("mode", ["thread", "warp", "fused"])
def test_true_classes_as_proposals_are_accepted_and_exact(lib, mode):
    torch = _torch()
    from ecmgenerator_gb300 import proposal as P

    a, b = _pair(mode=mode)
    accepted = proposed = 0
    for t in range(10):
        a.set_trace(True)
        a.update()
        _, y, slots = a.get_trace(device=True)
        cls = torch.full((a.max_agents,), P.CLS_OTHER, dtype=torch.uint8, device="cuda")
        cls[slots.long()] = y
        b.set_proposal_classes(cls)
        st = b.update()
        proposed += st.proposed
        accepted += st.accepted
        # the proposal path gives the plain LP's results bit for bit
        assert np.array_equal(a.get_position_data(), b.get_position_data()), t
        assert np.array_equal(a.get_velocity_data(), b.get_velocity_data()), t
    assert proposed > 0
    assert accepted >= 0.95 * proposed, (accepted, proposed)
    a.close()
    b.close()


@pytest.mark.parametrize("mode", ["thread", "warp", "fused"])
def test_wrong_proposals_are_rejected_and_results_unchanged(lib, mode):
    torch = _torch()

    a, b = _pair(mode=mode)
    g = torch.Generator(device="cuda").manual_seed(3)
    for t in range(10):
        a.update()
        cls = torch.randint(0, 153, (b.max_agents,), generator=g, device="cuda", dtype=torch.int32)
        b.set_proposal_classes(cls.to(torch.uint8).contiguous())
        b.update()
        assert np.array_equal(a.get_position_data(), b.get_position_data()), t
        assert np.array_equal(a.get_velocity_data(), b.get_velocity_data()), t
    a.close()
    b.close()


def test_trained_model_gains_over_untrained_and_constant(lib):
    """Ablation: acceptance rate (share of LPs whose incremental solve is
    skipped) of the trained network against an untrained one and against
    always proposing the most frequent class; trajectories stay those of the
    plain LP."""
    torch = _torch()
    from ecmgenerator_gb300 import proposal as P

    src = _c1_sim(seed=8)
    src.update(ticks=10)
    x, y = P.collect_traces(src, ticks=150)
    src.close()
    hist = P.class_histogram(y)
    assert hist["other"] < 0.9, hist
    model = P.ProposalModel(seed=2)
    model.train(x, y, steps=600, batch=8192, lr=2e-3, seed=5, log=False)
    untrained = P.ProposalModel(seed=2)
    major = int(torch.bincount(y[y != P.CLS_OTHER].long(), minlength=160).argmax())

    def run(setup):
        a, b = _pair(ticks=40)
        setup(b)
        acc = prop = 0
        for _ in range(40):
            a.update()
            st = b.update()
            acc += st.accepted
            prop += st.agent_steps
        ok = np.abs(a.get_position_data() - b.get_position_data()).max()
        a.close()
        b.close()
        return acc / max(prop, 1), ok

    def use(m):
        def f(s):
            s.set_proposal(m)
            s.set_proposal_gate(0.0, 0)  # model on every tick
        return f

    r_trained, d1 = run(use(model))
    r_untrained, d2 = run(use(untrained))
    r_const, d3 = run(lambda s: s.set_proposal_classes(
        torch.full((s.max_agents,), major, dtype=torch.uint8, device="cuda")))
    print(f"acceptance trained {r_trained:.3f} untrained {r_untrained:.3f} constant {r_const:.3f}; classes {hist}")
    assert max(d1, d2, d3) == 0.0  # accepted proposals give the plain LP's bits
    assert r_trained > r_untrained + 0.1
    assert r_trained > r_const + 0.05
    model.close()
    untrained.close()


def test_gate_pauses_a_model_that_is_rarely_accepted(lib):
    _torch()
    from ecmgenerator_gb300 import proposal as P

    a, b = _pair(ticks=5)
    m = P.ProposalModel(seed=9)
    b.set_proposal(m)
    b.set_proposal_gate(1.0, 3)  # no tick reaches 100 % acceptance: 1 model tick, 3 plain, ...
    st_b = b.update(ticks=8)
    a.update(ticks=8)
    assert st_b.gated == 6, st_b.gated
    assert np.array_equal(a.get_position_data(), b.get_position_data())
    b.set_proposal(None)
    a.close()
    b.close()
    m.close()

"""The adjoint of the trait peel.

sl_problem_trait_backward_eval (host, FP64) and sl_trait_backward (device,
FP32 with power-of-two rescaling) give d log L / d (theta_L, theta_R,
penetrance x3, disease-allele frequency) at every LOD position, L the
trait-peel likelihood of TraitRfunction's peel (trait_rfunction.cc:28-137,
peeler.cc:79-91).  The host gradient is checked here against central finite
differences of the oracle's FP64 LOD (which equals the reference's,
test_oracle_pin.py); the device gradient is checked against the host one.

Finite differences: central, step 1e-5 times the parameter's scale.  log L
behaves like r log(theta) and k log(q), and near a penetrance of 0 or 1 like
log(L0 + pen L1) with L1/L0 up to ~1e11 (recessive model, rare allele), so a
fixed absolute step would leave truncation error of order (h g)^2 or step
the likelihood through zero.  The scale is min(x, 1/(100 max|g|)) (x = 1 at a
penetrance of 0), max|g| the largest host gradient over the positions checked.
Tolerance: 1e-4 relative to the norm of the gradient over those positions.
"""
import ctypes

import numpy as np
import pytest

from conftest import CASES, load_golden
from swiftlink_gb300 import api
from swiftlink_gb300.workloads import disease_probs

FD_STEP = 1e-5
GRAD_RTOL = 1e-4
# a dominant, incompletely penetrant model next to the cases' recessive one
DOMINANT = ((0.01, 0.8, 0.9), 1e-3)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from swiftlink_gb300 import build
    build.build()


def with_model(g, pen, freq):
    d = dict(g)
    d["penetrance"] = np.array(pen, np.float64)
    d["freq"] = np.float64(freq)
    d["disease_prob"] = disease_probs(g["affection"], g["mother"] < 0, freq, pen)
    return d


def host_grad(d, dg, locus, offset):
    prob = api.Problem.from_arrays(d)
    desc = prob.desc()
    out = np.zeros(6)
    ptr = dg.ctypes.data_as(ctypes.c_void_p) if dg is not None else None
    rc = api.lib().sl_problem_trait_backward_eval(ctypes.byref(desc), ptr, int(locus), int(offset),
                                                 out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0, api.lib().sl_last_error(None)
    return out


def port_lod(d, dgs):
    from oracle import port
    raw, _, tp = port.Port(d).lod(dgs)
    return raw, tp


def fd_grads(d, dg, gmax, gtp):
    """Central differences of the oracle's per-position log L: returns
    dpartial [positions] (the derivative along partial theta of every
    interval, scaled by partial), and dmodel [4][positions], dtp [4].
    gmax[k], gtp[k]: the largest |d log L / d model parameter k| expected
    over the positions, and |d log P(T) / d parameter k|."""
    pen = np.array(d["penetrance"], np.float64)
    q = float(d["freq"])
    part = np.asarray(d["partial"], np.float64)
    hp = FD_STEP * part
    up, _ = port_lod(dict(d, partial=part + hp), dg[None])
    dn, _ = port_lod(dict(d, partial=part - hp), dg[None])
    dpartial = (up - dn) / 2.0           # = sum_k (dlogL/dtheta_k)(dtheta_k/dpartial) * hp
    dmodel, dtp = [], []
    for k in range(4):
        x = pen[k] if k < 3 else q
        for gm, out, j in ((gmax[k], dmodel, 0), (gtp[k], dtp, 1)):
            h = FD_STEP * min(abs(x) if x != 0.0 else 1.0, 1.0 / (100.0 * max(gm, 1e-30)))
            h = (x + h) - x          # a step that x + h and x - h represent exactly
            res = []
            for sgn in (1.0, -1.0):
                p2, q2 = pen.copy(), q
                if k < 3:
                    p2[k] += sgn * h
                else:
                    q2 += sgn * h
                # P(T) alone: no graph, so no position is evaluated at this step
                res.append(port_lod(with_model(d, p2, q2), dg[None] if j == 0 else dg[None][:0])[j])
            out.append((res[0] - res[1]) / (2 * h))
    return hp, dpartial, np.array(dmodel), np.array(dtp)


def sample_loci(M, seed):
    rng = np.random.default_rng(seed)
    return sorted(set([0, M - 2] + [int(x) for x in rng.integers(0, M - 1, 4)]))


@pytest.mark.parametrize("model", ["recessive", "dominant"])
@pytest.mark.parametrize("name", CASES)
def test_host_adjoint_matches_finite_differences(name, model):
    g = load_golden(name)
    d = g if model == "recessive" else with_model(g, *DOMINANT)
    n = g["n_lod"]
    dg = np.ascontiguousarray(g["lod_graphs"][-1], np.int32)
    pos = [(l, o) for l in sample_loci(g["M"], 5) for o in range(n)]
    grads = [host_grad(d, dg, l, o) for l, o in pos]
    gp = host_grad(d, None, 0, 0)   # log P(T): the peel with every recombination term 1/4
    gmax = np.abs(np.vstack(grads)[:, 2:]).max(axis=0)
    hp, dpart, dmodel, dtp = fd_grads(d, dg, gmax, np.abs(gp[2:]))
    want_t, got_t, want_m, got_m = [], [], [], []
    for (l, o), gr in zip(pos, grads):
        if True:
            i = l * n + o
            # theta_L = partial * (o+1), theta_R = partial * (n-o)
            got_t.append(hp[l] * ((o + 1) * gr[0] + (n - o) * gr[1]))
            want_t.append(dpart[i])
            got_m.append(gr[2:])
            want_m.append(dmodel[:, i])
    want_t, got_t = np.array(want_t), np.array(got_t)
    want_m, got_m = np.array(want_m), np.array(got_m)
    assert np.linalg.norm(got_t - want_t) <= GRAD_RTOL * np.linalg.norm(want_t) + 1e-9
    for k in range(4):
        scale = np.linalg.norm(want_m[:, k])
        err = np.linalg.norm(got_m[:, k] - want_m[:, k])
        assert err <= GRAD_RTOL * scale + 1e-9, (k, err, scale)
    np.testing.assert_allclose(gp[2:], dtp, rtol=GRAD_RTOL, atol=1e-9)


def test_theta_components_separately():
    """theta_L and theta_R through two offsets of one interval: the
    directional derivatives (o+1, n-o) at o = 0 and o = n-1 are independent."""
    g = load_golden("cfg1")
    n = g["n_lod"]
    dg = np.ascontiguousarray(g["lod_graphs"][1], np.int32)
    from oracle import port
    l = 37
    for o in (0, n - 1):
        gr = host_grad(g, dg, l, o)
        base = float(g["partial"][l])
        h = FD_STEP * base
        ups = []
        for sgn in (1.0, -1.0):
            part = np.array(g["partial"], np.float64)
            part[l] = base + sgn * h
            raw, _, _ = port.Port(dict(g, partial=part)).lod(dg[None])
            ups.append(raw[l * n + o])
        fd = (ups[0] - ups[1]) / (2 * h)
        an = (o + 1) * gr[0] + (n - o) * gr[1]
        assert abs(fd - an) <= GRAD_RTOL * max(1.0, abs(fd)), (o, fd, an)


# ---------------------------------------------------------------- device ----

def host_all(d, dg, positions):
    return np.array([host_grad(d, dg, l, o) for l, o in positions])


def rel_err(got, want):
    return np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300)


# shared bytes per task: 0 = the default plan (every rfunction kept on these
# pedigrees), 256 = below any plan, so the smallest split into segments with
# recomputation is taken
BUDGETS = [0, 256]


@pytest.mark.gpu
@pytest.mark.parametrize("budget", BUDGETS)
@pytest.mark.parametrize("model", ["recessive", "dominant"])
@pytest.mark.parametrize("name", CASES)
def test_device_adjoint_matches_host_fp64(name, model, budget):
    """FP32 device adjoint with rescaling against the FP64 host adjoint, every
    position of every golden graph, each of the six components within 1e-4
    of its norm; d log P(T) within 1e-4 relative -- with every rfunction kept
    and with the forward cutsets recomputed segment by segment."""
    g = load_golden(name)
    d = g if model == "recessive" else with_model(g, *DOMINANT)
    n = g["n_lod"]
    graphs = np.ascontiguousarray(g["lod_graphs"], np.int32)
    with api.Context(api.Problem.from_arrays(d), n_chains=1) as ctx:
        seg, used = ctx.adjoint_memory(budget)
        assert (seg == 1) == (budget == 0), (seg, used)
        grad, pt = ctx.trait_backward(graphs)
    positions = [(l, o) for l in range(g["M"] - 1) for o in range(n)]
    for b in range(graphs.shape[0]):
        want = host_all(d, graphs[b], positions)
        got = grad[b].reshape(-1, 6)
        for k in range(6):
            assert rel_err(got[:, k], want[:, k]) <= GRAD_RTOL, (b, k, rel_err(got[:, k], want[:, k]))
    want_pt = host_grad(d, None, 0, 0)[2:]
    np.testing.assert_allclose(pt, want_pt, rtol=GRAD_RTOL)


@pytest.mark.gpu
@pytest.mark.parametrize("budget", BUDGETS)
def test_device_adjoint_large_pedigree(budget):
    """The 120-member, 2000-SNP pedigree under the dominant model: the device
    adjoint of its starting graph at sampled positions against the host, with
    every rfunction kept (the default plan here) and recomputed."""
    from swiftlink_gb300.workloads import load_problem
    g = load_problem("cfg2")
    d = with_model(g, *DOMINANT)
    n = g["n_lod"]
    dg = np.ascontiguousarray(g["dg0"], np.int32)
    with api.Context(api.Problem.from_arrays(d), n_chains=1) as ctx:
        seg, used = ctx.adjoint_memory(budget)
        assert (seg == 1) == (budget == 0), (seg, used)
        grad, pt = ctx.trait_backward(dg[None])
    positions = [(l, o) for l in sample_loci(g["M"], 9) for o in range(n)]
    want = host_all(d, dg, positions)
    got = np.array([grad[0, l, o] for l, o in positions])
    for k in range(6):
        assert rel_err(got[:, k], want[:, k]) <= GRAD_RTOL, (k, rel_err(got[:, k], want[:, k]))
    np.testing.assert_allclose(pt, host_grad(d, None, 0, 0)[2:], rtol=GRAD_RTOL)


@pytest.mark.gpu
def test_device_adjoint_400_member_pedigree_recomputes():
    """The 400-member, 10,000-SNP pedigree under the dominant model: its
    dense rfunctions and adjoints (about 92 KB per task) exceed the default
    budget, so the default plan splits the peel into segments and
    recomputes; the device adjoint of the starting graph at sampled positions
    against the host FP64 adjoint (which rescales too: the plain peel
    underflows here); the plan needs less than half the dense footprint.
    Its cutsets of five members rule out the compiled form."""
    from swiftlink_gb300 import pedigree, synth
    g = pedigree.problem_from_workload(synth.make_workload(5))
    d = with_model(g, *DOMINANT)
    n = g["n_lod"]
    dg = np.ascontiguousarray(g["dg0"], np.int32)
    with api.Context(api.Problem.from_arrays(d), n_chains=1) as ctx:
        seg, used = ctx.adjoint_memory(0)
        dense = 8 * sum(4 ** len(c) for c in g["op_cutset"])   # every matrix and its adjoint, FP32
        assert seg > 1 and used < dense // 2, (seg, used, dense)
        with pytest.raises(api.SwiftLinkError):
            ctx.adjoint_set_form(api.SL_ADJOINT_SPECIALISED)
        grad, pt = ctx.trait_backward(dg[None])
        assert ctx.adjoint_info()[0] in (api.SL_ADJOINT_WARP, api.SL_ADJOINT_THREAD)
    positions = [(l, o) for l in sample_loci(g["M"], 5) for o in range(n)]
    want = host_all(d, dg, positions)
    got = np.array([grad[0, l, o] for l, o in positions])
    for k in range(6):
        assert rel_err(got[:, k], want[:, k]) <= GRAD_RTOL, (k, rel_err(got[:, k], want[:, k]))
    np.testing.assert_allclose(pt, host_grad(d, None, 0, 0)[2:], rtol=GRAD_RTOL)


FORMS = [(api.SL_ADJOINT_WARP, 0), (api.SL_ADJOINT_THREAD, 0)] + \
    [(api.SL_ADJOINT_SPECIALISED, v) for v in range(api.SL_ADJOINT_VARIANTS)]


@pytest.mark.gpu
@pytest.mark.parametrize("form,variant", FORMS)
@pytest.mark.parametrize("model", ["recessive", "dominant"])
@pytest.mark.parametrize("name", CASES)
def test_each_adjoint_form_matches_host_fp64(name, model, form, variant):
    """Each form fixed by sl_adjoint_set_form -- the warp form, the thread
    form and every variant of the peel's adjoint compiled for the pedigree --
    against the FP64 host adjoint at every position of every golden graph."""
    g = load_golden(name)
    d = g if model == "recessive" else with_model(g, *DOMINANT)
    n = g["n_lod"]
    graphs = np.ascontiguousarray(g["lod_graphs"], np.int32)
    with api.Context(api.Problem.from_arrays(d), n_chains=1) as ctx:
        ctx.adjoint_set_form(form, variant)
        grad, _ = ctx.trait_backward(graphs)
        assert ctx.adjoint_info()[0] == form
        if form == api.SL_ADJOINT_SPECIALISED:
            shapes, used, regs, ms = ctx.adjoint_kernel_info()
            assert shapes >= 1 and used == variant and regs > 0 and ms > 0
    positions = [(l, o) for l in range(g["M"] - 1) for o in range(n)]
    for b in range(graphs.shape[0]):
        want = host_all(d, graphs[b], positions)
        got = grad[b].reshape(-1, 6)
        for k in range(6):
            assert rel_err(got[:, k], want[:, k]) <= GRAD_RTOL, (b, k, rel_err(got[:, k], want[:, k]))


@pytest.mark.gpu
def test_specialised_adjoint_large_pedigree_and_timed_choice():
    """The 120-member, 2000-SNP pedigree under the dominant model: the
    compiled adjoint of its starting graph at sampled positions against the
    host; the timed choice then covers all three forms.  Under a plan that
    splits the peel the compiled form (which keeps every rfunction) is
    refused and left out of the timing."""
    from swiftlink_gb300.workloads import load_problem
    g = load_problem("cfg2")
    d = with_model(g, *DOMINANT)
    n = g["n_lod"]
    dg = np.ascontiguousarray(g["dg0"], np.int32)
    positions = [(l, o) for l in sample_loci(g["M"], 11) for o in range(n)]
    want = host_all(d, dg, positions)
    with api.Context(api.Problem.from_arrays(d), n_chains=1) as ctx:
        ctx.adjoint_set_form(api.SL_ADJOINT_SPECIALISED)
        grad, _ = ctx.trait_backward(dg[None])
        got = np.array([grad[0, l, o] for l, o in positions])
        for k in range(6):
            assert rel_err(got[:, k], want[:, k]) <= GRAD_RTOL, (k, rel_err(got[:, k], want[:, k]))
        ctx.adjoint_set_form(0)
        grad, _ = ctx.trait_backward(dg[None])
        form, warp_ms, thread_ms, spec_ms = ctx.adjoint_info()
        assert warp_ms > 0 and thread_ms > 0 and spec_ms > 0
        assert form in (api.SL_ADJOINT_WARP, api.SL_ADJOINT_THREAD, api.SL_ADJOINT_SPECIALISED)
        got = np.array([grad[0, l, o] for l, o in positions])   # the form (and register budget) timing kept
        for k in range(6):
            assert rel_err(got[:, k], want[:, k]) <= GRAD_RTOL, (k, rel_err(got[:, k], want[:, k]))
        seg, _ = ctx.adjoint_memory(256)
        assert seg > 1
        with pytest.raises(api.SwiftLinkError):
            ctx.adjoint_set_form(api.SL_ADJOINT_SPECIALISED)
        ctx.trait_backward(dg[None])
        form, warp_ms, thread_ms, spec_ms = ctx.adjoint_info()
        assert spec_ms == 0 and form in (api.SL_ADJOINT_WARP, api.SL_ADJOINT_THREAD)


@pytest.mark.gpu
def test_autograd_function_wrapper_matches_finite_differences():
    """The C-ABI backward behind a torch.autograd.Function (test harness only):
    log L [G][M-1][n] as a function of partial theta [M-1], the penetrances
    [3] and the disease-allele frequency, forward by the FP64 device LOD,
    backward by sl_trait_backward; a weighted loss differentiated through it
    equals its central finite differences."""
    torch = pytest.importorskip("torch")
    g0 = load_golden("cfg1")
    n, M = g0["n_lod"], g0["M"]
    graphs = np.ascontiguousarray(g0["lod_graphs"], np.int32)

    def problem(partial, pen, q):
        d = with_model(g0, pen, q)
        d["partial"] = partial
        return d

    def forward_np(partial, pen, q):
        out = []
        with api.Context(api.Problem.from_arrays(problem(partial, pen, q)), n_chains=1) as ctx:
            for b in range(graphs.shape[0]):
                ctx.lod_reset()
                ctx.lod_score_graphs(graphs[b:b + 1])
                raw, _, _ = ctx.lod_results()
                out.append(raw.reshape(M - 1, n))
        return np.stack(out)

    class TraitPeel(torch.autograd.Function):
        @staticmethod
        def forward(fctx, partial, pen, q):
            args = (partial.detach().numpy(), pen.detach().numpy(), float(q))
            fctx.args = args
            return torch.from_numpy(forward_np(*args))

        @staticmethod
        def backward(fctx, gout):
            partial, pen, q = fctx.args
            with api.Context(api.Problem.from_arrays(problem(partial, pen, q)), n_chains=1) as ctx:
                grad, _ = ctx.trait_backward(graphs)
            go = gout.detach().numpy()[..., None]                      # [G][M-1][n][1]
            o = np.arange(n)
            dpart = (go[..., 0] * ((o + 1) * grad[..., 0] + (n - o) * grad[..., 1])).sum(axis=(0, 2))
            dmodel = (go * grad[..., 2:]).sum(axis=(0, 1, 2))
            return (torch.from_numpy(dpart), torch.from_numpy(dmodel[:3]),
                    torch.tensor(dmodel[3], dtype=torch.float64))

    pen0, q0 = DOMINANT
    partial = torch.tensor(np.asarray(g0["partial"], np.float64), requires_grad=True)
    pen = torch.tensor(pen0, dtype=torch.float64, requires_grad=True)
    q = torch.tensor(q0, dtype=torch.float64, requires_grad=True)
    w = torch.from_numpy(np.random.default_rng(2).random((graphs.shape[0], M - 1, n)))
    loss = (TraitPeel.apply(partial, pen, q) * w).sum()
    loss.backward()

    def loss_at(partial_np, pen_np, q_np):
        return float((forward_np(partial_np, pen_np, q_np) * w.numpy()).sum())

    base_part = np.asarray(g0["partial"], np.float64)
    # partial theta: a random direction, relative step
    rng = np.random.default_rng(4)
    v = rng.standard_normal(M - 1) * base_part
    h = FD_STEP
    fd = (loss_at(base_part + h * v, np.array(pen0), q0) - loss_at(base_part - h * v, np.array(pen0), q0)) / (2 * h)
    an = float(partial.grad.numpy() @ v)
    assert abs(fd - an) <= GRAD_RTOL * max(abs(fd), 1.0), (fd, an)
    for k in range(4):
        x = pen0[k] if k < 3 else q0
        hk = FD_STEP * x
        hk = (x + hk) - x
        vals = []
        for sgn in (1.0, -1.0):
            p2, q2 = np.array(pen0, np.float64), q0
            if k < 3:
                p2[k] += sgn * hk
            else:
                q2 += sgn * hk
            vals.append(loss_at(base_part, p2, q2))
        fdk = (vals[0] - vals[1]) / (2 * hk)
        ank = float(pen.grad[k]) if k < 3 else float(q.grad)
        assert abs(fdk - ank) <= GRAD_RTOL * max(abs(fdk), 1.0), (k, fdk, ank)

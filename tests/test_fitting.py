"""Gradients of the Tersoff fitting workload (energies and forces of a batch
of diamond Si supercells as functions of the 14 continuous parameters and of
the positions) against central finite differences: of the GPU's own FP64
energies (h = 1e-6 relative; absolute for mubo, whose value is 0), of the
oracle's energies (the reference algorithm), and, for the loss, through
torch.autograd."""

import numpy as np
import pytest

import oracle
from atomistica_gb300 import structures as S

pytestmark = pytest.mark.gpu


def _setup(n=6, seed=51):
    from atomistica_gb300 import fitting
    structs = S.si_fit_set(n, seed=seed)
    theta, m = fitting.single_element_parameters()
    return fitting, structs, fitting.TersoffBatch(structs, m=m), theta, m


def _step(theta, k):
    return 1e-6 * abs(theta[k]) if theta[k] != 0.0 else 1e-6


def test_values_match_oracle(gpu):
    fitting, structs, tb, theta, m = _setup()
    e, _, f, _ = tb.evaluate(theta)
    params = fitting.parameter_dict(theta, m)
    for q, s in enumerate(structs):
        ref = oracle.bop("tersoff", params, s, per_at=False)
        assert abs(e[q] - ref["epot"]) / len(s) < 1e-10
        assert np.max(np.abs(f[tb.offsets[q]:tb.offsets[q + 1]] - ref["f"])) < 1e-9


def test_parameter_tangents_match_central_differences(gpu):
    fitting, structs, tb, theta, m = _setup()
    for k, name in enumerate(fitting.PARAM_NAMES):
        u = np.zeros(14)
        u[k] = 1.0
        _, de, _, df = tb.evaluate(theta, dtheta=u)
        h = _step(theta, k)
        ep, _, fp, _ = tb.evaluate(theta + h * u)
        em, _, fm, _ = tb.evaluate(theta - h * u)
        fd_e = (ep - em) / (2 * h)
        fd_f = (fp - fm) / (2 * h)
        scale_e = max(np.max(np.abs(de)), 1e-300)
        assert np.max(np.abs(de - fd_e)) <= 1e-6 * scale_e, (name, de, fd_e)
        scale_f = max(np.max(np.abs(df)), 1e-300)
        assert np.max(np.abs(df - fd_f)) <= 1e-5 * scale_f, name


def test_parameter_tangents_match_oracle_differences(gpu):
    # finite differences of the reference algorithm's own energies
    fitting, structs, tb, theta, m = _setup(3, seed=52)
    for k, name in enumerate(fitting.PARAM_NAMES):
        u = np.zeros(14)
        u[k] = 1.0
        _, de, _, _ = tb.evaluate(theta, dtheta=u)
        h = _step(theta, k)
        pp = fitting.parameter_dict(theta + h * u, m)
        pm = fitting.parameter_dict(theta - h * u, m)
        for q, s in enumerate(structs):
            fd = (oracle.bop("tersoff", pp, s, per_at=False)["epot"] -
                  oracle.bop("tersoff", pm, s, per_at=False)["epot"]) / (2 * h)
            assert abs(de[q] - fd) <= 1e-6 * max(abs(de[q]), abs(fd)) + 1e-9 * len(s), \
                (name, q, de[q], fd)


def test_hessian_vector_product(gpu):
    fitting, structs, tb, theta, m = _setup(4, seed=53)
    r0 = np.concatenate([s.positions for s in structs])
    rng = np.random.default_rng(7)
    v = rng.normal(size=r0.shape)
    tb.set_positions(r0)
    _, de, f, hv = tb.evaluate(theta, dr=v)
    # dE along v = -F . v (per structure)
    for q in range(len(structs)):
        sl = slice(tb.offsets[q], tb.offsets[q + 1])
        assert abs(de[q] + np.sum(f[sl] * v[sl])) <= 1e-9 * max(1.0, abs(de[q]))
    eps = 1e-5
    tb.set_positions(r0 + eps * v)
    _, _, fp, _ = tb.evaluate(theta)
    tb.set_positions(r0 - eps * v)
    _, _, fm, _ = tb.evaluate(theta)
    fd = (fp - fm) / (2 * eps)
    assert np.max(np.abs(hv - fd)) <= 1e-6 * np.max(np.abs(hv))


def test_autograd_loss_gradients(gpu):
    torch = pytest.importorskip("torch")
    fitting, structs, tb, theta, m = _setup(4, seed=54)
    rng = np.random.default_rng(8)
    theta_t = theta * (1.0 + rng.uniform(-0.02, 0.02, size=14))  # targets: perturbed set
    theta_t[13] = 0.0
    r0 = np.concatenate([s.positions for s in structs])
    tb.set_positions(r0)
    et, _, ft, _ = tb.evaluate(theta_t)
    E_t, F_t = torch.tensor(et), torch.tensor(ft)

    def loss_of(th, r):
        E, F = fitting.EnergyForces.apply(th, r, tb)
        return fitting.fitting_loss(E, F, tb.nat, E_t, F_t)

    th = torch.tensor(theta, requires_grad=True)
    r = torch.tensor(r0, requires_grad=True)
    loss = loss_of(th, r)
    loss.backward()
    g_th, g_r = th.grad.numpy(), r.grad.numpy()
    with torch.no_grad():
        for k in range(14):
            h = _step(theta, k)
            u = torch.zeros(14, dtype=torch.float64)
            u[k] = h
            fd = (loss_of(th.detach() + u, r.detach()) -
                  loss_of(th.detach() - u, r.detach())).item() / (2 * h)
            assert abs(g_th[k] - fd) <= 1e-6 * max(abs(g_th[k]), abs(fd)) + 1e-12, \
                (fitting.PARAM_NAMES[k], g_th[k], fd)
        v = torch.tensor(rng.normal(size=r0.shape))
        eps = 1e-5
        fd = (loss_of(th.detach(), r.detach() + eps * v) -
              loss_of(th.detach(), r.detach() - eps * v)).item() / (2 * eps)
        ana = float(np.sum(g_r * v.numpy()))
        assert abs(ana - fd) <= 1e-6 * max(abs(ana), abs(fd)) + 1e-12


def test_adjoint_matches_tangents(gpu):
    # the reverse-mode pass against the forward-mode tangents (one per
    # parameter), value part and derivative along v, at 1e-10 relative
    fitting, structs, tb, theta, m = _setup(5, seed=55)
    r0 = np.concatenate([s.positions for s in structs])
    tb.set_positions(r0)
    v = np.random.default_rng(9).normal(size=r0.shape)
    e, f, hv, g, gd = tb.adjoint(theta, v)
    e0, _, f0, hv0 = tb.evaluate(theta, dr=v)
    assert np.max(np.abs(e - e0)) <= 1e-12 * np.max(np.abs(e0))
    assert np.max(np.abs(f - f0)) <= 1e-12 * np.max(np.abs(f0))
    assert np.max(np.abs(hv - hv0)) <= 1e-12 * np.max(np.abs(hv0))
    for k, name in enumerate(fitting.PARAM_NAMES):
        u = np.zeros(14)
        u[k] = 1.0
        _, de, _, df = tb.evaluate(theta, dtheta=u)
        # D_v(dE_s/dtheta_k) = -sum_{i in s} v_i . dF_i/dtheta_k
        dv = np.array([-np.sum(v[tb.offsets[q]:tb.offsets[q + 1]] *
                               df[tb.offsets[q]:tb.offsets[q + 1]])
                       for q in range(len(structs))])
        assert np.max(np.abs(g[:, k] - de)) <= 1e-10 * max(np.max(np.abs(de)), 1e-300), \
            (name, g[:, k], de)
        assert np.max(np.abs(gd[:, k] - dv)) <= 1e-10 * max(np.max(np.abs(dv)), 1e-300), \
            (name, gd[:, k], dv)


def test_adjoint_matches_central_differences(gpu):
    # dE/dtheta of the adjoint against central differences of the energies
    fitting, structs, tb, theta, m = _setup(4, seed=56)
    _, _, _, g, _ = tb.adjoint(theta)
    for k, name in enumerate(fitting.PARAM_NAMES):
        u = np.zeros(14)
        u[k] = 1.0
        h = _step(theta, k)
        ep, _, _, _ = tb.evaluate(theta + h * u)
        em, _, _, _ = tb.evaluate(theta - h * u)
        fd = (ep - em) / (2 * h)
        assert np.max(np.abs(g[:, k] - fd)) <= 1e-6 * max(np.max(np.abs(g[:, k])), 1e-300), \
            (name, g[:, k], fd)


def test_sharded_path_equals_autograd(gpu):
    # fitting.sharded_loss_and_gradient (the multi-rank path; world size 1
    # here) on the GPU batch equals the torch.autograd path
    torch = pytest.importorskip("torch")
    fitting, structs, tb, theta, m = _setup(4, seed=57)
    rng = np.random.default_rng(10)
    theta_t = theta * (1.0 + rng.uniform(-0.02, 0.02, size=14))
    r0 = np.concatenate([s.positions for s in structs])
    tb.set_positions(r0)
    et, _, ft, _ = tb.evaluate(theta_t)
    tb.set_positions(r0)
    loss, g, gp = fitting.sharded_loss_and_gradient(theta, tb, tb.nat, et, ft)
    th = torch.tensor(theta, requires_grad=True)
    r = torch.tensor(r0, requires_grad=True)
    E, F = fitting.EnergyForces.apply(th, r, tb)
    L = fitting.fitting_loss(E, F, tb.nat, torch.tensor(et), torch.tensor(ft))
    L.backward()
    assert abs(loss - L.item()) <= 1e-13 * abs(L.item())
    assert np.max(np.abs(g - th.grad.numpy())) <= 1e-12 * np.max(np.abs(g))
    assert np.max(np.abs(gp - r.grad.numpy())) <= 1e-12 * np.max(np.abs(gp))

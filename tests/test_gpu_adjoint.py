"""The hand-written adjoint of the condensation sub-steps (k_adjoint.cu,
adjoint.py) against central finite differences of its own forward model in
FP64: d LWP / d kappa and d LWP / d m_s of single SIPs, and checkpointed
against single-segment gradients."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lacmopy_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def model():
    from lacmopy_gb300 import adjoint, synthetic
    st = synthetic.make_icmw_state(Nx=3, Nz=75, seed=7, kernel_type="Long_Bott")
    return adjoint.CondensationModel(st)


N_SUB = 20


def _J(model, m_s, kappa):
    m_w, _, _ = model.run(m_s, kappa, N_SUB)
    return float((model.lwp_weights() * m_w).sum())


def test_gradients_vs_finite_differences(model):
    from lacmopy_gb300 import adjoint
    m_s = model.m_s0.clone().requires_grad_(True)
    kappa = torch.tensor(0.6, dtype=torch.float64, device="cuda", requires_grad=True)
    J = adjoint.liquid_water(model, m_s, kappa, n_sub=N_SUB, checkpoint_every=7)
    J.backward()
    assert abs(float(J.detach()) - _J(model, model.m_s0, 0.6)) <= 1e-14 * abs(float(J.detach()))
    # kappa
    h = 1e-5
    fd = (_J(model, model.m_s0, 0.6 + h) - _J(model, model.m_s0, 0.6 - h)) / (2 * h)
    assert fd != 0.0
    assert abs(float(kappa.grad) - fd) <= 2e-5 * abs(fd)
    # solute masses of single SIPs whose perturbation moves J well above the
    # rounding noise of J (the per-cell sums are atomics in arbitrary order)
    g = m_s.grad.cpu().numpy()
    cell = model.cell.cpu().numpy()
    ms0 = model.m_s0.cpu().numpy()
    order = np.argsort(-np.abs(g * ms0))
    picks = list(order[:3]) + list(order[100:102]) + list(order[1000:1002])
    for k in picks:
        base = model.m_s0.clone()
        hk = 1e-4 * float(base[k])
        up, dn = base.clone(), base.clone()
        up[k] += hk
        dn[k] -= hk
        fdk = (_J(model, up, 0.6) - _J(model, dn, 0.6)) / (2 * hk)
        assert cell[k] >= 0
        assert abs(g[k] - fdk) <= 1e-3 * abs(fdk) + 1e-6 * np.abs(g).max(), (k, g[k], fdk)


def test_checkpointing_does_not_change_gradients(model):
    from lacmopy_gb300 import adjoint
    out = []
    for every in (4, N_SUB):
        m_s = model.m_s0.clone().requires_grad_(True)
        kappa = torch.tensor(0.6, dtype=torch.float64, device="cuda", requires_grad=True)
        adjoint.liquid_water(model, m_s, kappa, n_sub=N_SUB, checkpoint_every=every).backward()
        out.append((m_s.grad.clone(), float(kappa.grad)))
    torch.testing.assert_close(out[0][0], out[1][0], rtol=1e-9, atol=1e-30)
    assert abs(out[0][1] - out[1][1]) <= 1e-9 * abs(out[1][1])

"""The hand-written adjoint (k_adjoint.cu, adjoint.py) in FP64.

Condensation model: d LWP / d kappa and d LWP / d m_s of single SIPs against
central finite differences of its own forward model, checkpointed against
single-segment gradients.  Step model (the product's step replayed with
recorded cells): the forward against the product's own run, gradients of the
liquid water path and the surface rain by kappa, the mass-flux scale and m_s
against finite differences and against autograd through an FP64 PyTorch
restatement, checkpoint invariance, and the converged-root gradient against the
time step's own 3-evaluation Newton map."""
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


# ---- the step model: the product's time step replayed with recorded cells ----
N_ADV = 30   # long enough for drizzle drops to reach the ground


@pytest.fixture(scope="module")
def step_model():
    from lacmopy_gb300 import adjoint, synthetic
    st = synthetic.make_icmw_state(Nx=8, Nz=10, no_spcm=(6, 8), seed=11, kernel_type="Long_Bott",
                                   drizzle_fraction=0.3, r_tot=12.5E-3)
    return st, adjoint.StepModel(st, N_ADV)


def test_step_model_replays_the_product_run(step_model):
    """With the recorded cells and collisions the forward model is the
    product's FP64 step: the same masses, multiplicities, Theta, r_v and
    surface rain."""
    st, model = step_model
    m_w, m_s, xi, Th, rv = model.run(full=True)
    ds = model.product
    mw_p = ds.m_w
    assert model.cells.min() < 0 <= model.cells.max()
    assert model.n_events > 0   # collisions replayed
    torch.testing.assert_close(m_w, mw_p, rtol=1e-11, atol=1e-30)
    torch.testing.assert_close(m_s, ds.m_s, rtol=1e-12, atol=0)
    torch.testing.assert_close(xi, ds.xi, rtol=1e-12, atol=0)
    torch.testing.assert_close(Th, ds.gsf[2].reshape(-1), rtol=1e-13, atol=0)
    torch.testing.assert_close(rv, ds.gsf[4].reshape(-1), rtol=1e-11, atol=0)
    removed = model.rain_weights() > 0
    rain = float((m_w * model.xi)[removed].sum())
    rain_p = float(ds.water_removed[0]) - float(np.asarray(st["water_removed"])[0])
    assert removed.any() and abs(rain - rain_p) <= 1e-11 * abs(rain_p)


def _step_J(model, weights, m_s=None, kappa=0.6, s=1.0, no_iter=None):
    m_w, _, _ = model.run(m_s, kappa, s, no_iter)
    return float((weights * m_w).sum())


@pytest.mark.parametrize("target", ["lwp", "rain"])
def test_step_gradients_vs_finite_differences(step_model, target):
    from lacmopy_gb300 import adjoint
    _, model = step_model
    w = model.lwp_weights() if target == "lwp" else model.rain_weights()
    m_s = model.m_s0.clone().requires_grad_(True)
    kappa = torch.tensor(0.6, dtype=torch.float64, device="cuda", requires_grad=True)
    s = torch.tensor(1.0, dtype=torch.float64, device="cuda", requires_grad=True)
    J = adjoint.objective(model, m_s, kappa, s, weights=w, checkpoint_every=4)
    J.backward()
    assert abs(float(J.detach()) - _step_J(model, w)) <= 1e-13 * abs(float(J.detach()))
    # J is smooth between the map's floors and damping switches; the
    # exact-derivative check is the autograd comparison below
    h = 1e-4
    fd_k = (_step_J(model, w, kappa=0.6 + h) - _step_J(model, w, kappa=0.6 - h)) / (2 * h)
    fd_s = (_step_J(model, w, s=1.0 + h) - _step_J(model, w, s=1.0 - h)) / (2 * h)
    assert fd_k != 0.0 and fd_s != 0.0
    assert abs(float(kappa.grad) - fd_k) <= 1e-3 * abs(fd_k), (float(kappa.grad), fd_k)
    assert abs(float(s.grad) - fd_s) <= 1e-3 * abs(fd_s), (float(s.grad), fd_s)
    g = m_s.grad.cpu().numpy()
    ms0 = model.m_s0.cpu().numpy()
    order = np.argsort(-np.abs(g * ms0))
    for k in list(order[:3]) + list(order[50:52]):
        hk = 1e-4 * float(ms0[k])
        up, dn = model.m_s0.clone(), model.m_s0.clone()
        up[k] += hk
        dn[k] -= hk
        fdk = (_step_J(model, w, m_s=up) - _step_J(model, w, m_s=dn)) / (2 * hk)
        assert abs(g[k] - fdk) <= 1e-3 * abs(fdk) + 1e-6 * np.abs(g).max(), (k, g[k], fdk)


def test_step_gradients_vs_torch_fp64_autograd():
    """The hand-written adjoint against autograd through an FP64 PyTorch
    restatement of the same model (tests/torch_step_model.py) on the CPU,
    collisions replayed in both."""
    import torch_step_model as ref
    from lacmopy_gb300 import adjoint, synthetic
    st = synthetic.make_icmw_state(Nx=4, Nz=6, no_spcm=(3, 4), seed=5, kernel_type="Long_Bott",
                                   drizzle_fraction=0.3, r_tot=12.5E-3)
    st["dt_col_over_dV"] = 60.0 / st["grid_volume_cell"]   # collisions within two steps
    n_adv = 2
    model = adjoint.StepModel(st, n_adv)
    assert model.n_events > 0
    gen = torch.Generator().manual_seed(3)
    w = torch.rand(model.n, generator=gen, dtype=torch.float64)
    m_s = model.m_s0.clone().requires_grad_(True)
    kappa = torch.tensor(0.6, dtype=torch.float64, device="cuda", requires_grad=True)
    s = torch.tensor(1.0, dtype=torch.float64, device="cuda", requires_grad=True)
    J = adjoint.objective(model, m_s, kappa, s, weights=w.cuda())
    J.backward()
    m_s_r = torch.as_tensor(st["m_s"], dtype=torch.float64).clone().requires_grad_(True)
    kappa_r = torch.tensor(0.6, dtype=torch.float64, requires_grad=True)
    s_r = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    m_w_r = ref.run(st, model.cells.cpu(), m_s_r, kappa_r, s_r, n_adv, 3,
                    events=ref.decode_events(model.events))
    J_r = (w * m_w_r).sum()
    J_r.backward()
    assert abs(float(J.detach()) - float(J_r.detach())) <= 1e-12 * abs(float(J_r.detach()))
    gm, gr = m_s.grad.cpu(), m_s_r.grad
    assert float((gm - gr).abs().max()) <= 1e-7 * float(gr.abs().max())
    assert abs(float(kappa.grad) - float(kappa_r.grad)) <= 1e-7 * abs(float(kappa_r.grad))
    assert abs(float(s.grad) - float(s_r.grad)) <= 1e-7 * abs(float(s_r.grad))


def test_step_checkpointing_and_converged_root(step_model):
    """Checkpoint spacing does not change the gradient; the converged-root
    model's gradient (implicit-function theorem) stays close to that of the
    time step's own 3-evaluation map."""
    from lacmopy_gb300 import adjoint
    _, model = step_model
    out = {}
    for key, every, ni in (("c1", 1, None), ("cN", N_ADV, None), ("root", 3, 0)):
        m_s = model.m_s0.clone().requires_grad_(True)
        kappa = torch.tensor(0.6, dtype=torch.float64, device="cuda", requires_grad=True)
        s = torch.tensor(1.0, dtype=torch.float64, device="cuda", requires_grad=True)
        adjoint.objective(model, m_s, kappa, s, no_iter=ni, checkpoint_every=every).backward()
        out[key] = (m_s.grad.clone(), float(kappa.grad), float(s.grad))
    torch.testing.assert_close(out["c1"][0], out["cN"][0], rtol=1e-9, atol=1e-30)
    assert abs(out["c1"][1] - out["cN"][1]) <= 1e-9 * abs(out["cN"][1])
    assert abs(out["c1"][2] - out["cN"][2]) <= 1e-9 * abs(out["cN"][2])
    # converged root vs the 3-evaluation map
    assert abs(out["root"][1] - out["c1"][1]) <= 2e-2 * abs(out["c1"][1]), (out["root"][1], out["c1"][1])
    assert abs(out["root"][2] - out["c1"][2]) <= 2e-2 * abs(out["c1"][2]), (out["root"][2], out["c1"][2])

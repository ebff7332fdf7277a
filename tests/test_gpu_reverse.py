"""Reverse mode (des_adjoint_forward / des_adjoint_backward) against central
finite differences of the forward window, on small meshes.

The loss is linear in the final state, L = <seed, S_K> over coordinates,
velocities, temperature, stress and plastic strain, so its adjoint is the
seed.  For a direction d in the start state or in the parameters, the
adjoint's <adjoint, d> must equal (L(p + d) - L(p - d)) / 2.  Directions
are scaled to ~1e-6 of each field, so the central difference is accurate
to ~1e-9 where the step is smooth; the kinks of the forward (yield, the
EVP choice, viscosity clamps) are stepped over only where they are not
met within the perturbation.  Damping option 2 (continuous) is used: with
option 1 the step is discontinuous in the velocity sign.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("coord", "vel", "temperature", "stress", "plstrain")


def _window(wl, K, C, spin=4):
    from dynearthsol_gb300.adjoint import Window
    from dynearthsol_gb300.config import initial_state
    from dynearthsol_gb300.solver import DeviceModel
    st, cp = initial_state(wl)
    m = DeviceModel(wl, comp_pressure=cp)
    m.init_fields(st)
    if spin:
        m.step(spin)   # nonzero velocities and deviatoric stresses
    return Window(m, m.download(), m.clock(), K, C)


def _workload(name="c1_3d_evp", cells=(3, 3, 2), **params):
    from dataclasses import replace
    from dynearthsol_gb300.config import make_workload
    wl = make_workload(name, cells=cells)
    wl.params = replace(wl.params, damping_option=2, **params)
    return wl


def _seed(win, rng):
    final = win.run()
    seed = {}
    for k in FIELDS:
        a = final[k]
        sc = max(float(np.abs(a).max()), 1e-30)
        seed[k] = rng.standard_normal(a.shape) / sc
    return seed


def _dstate(win, rng, field, scale=1e-6):
    s = win.start
    a = s[field]
    if field == "coord":
        ext = s["coord"].max(axis=0) - s["coord"].min(axis=0)
        d = rng.standard_normal(a.shape) * (ext / 10)
    elif field == "plstrain":
        d = np.where(a > 1e-3, rng.standard_normal(a.shape) * np.maximum(a, 1e-3), 0.0)
    elif field == "volume_old":
        # vol / vol_old - 1 moves by the relative step (its rounding, 1e-16,
        # is the difference's floor) and the pressure by K times it (~500 Pa
        # at 1e-8; the deviators, and so the EVP choice, do not move)
        d = rng.standard_normal(a.shape) * a * (1e-8 / scale)
    else:
        d = rng.standard_normal(a.shape) * max(float(np.abs(a).max()), 1e-30)
    return {field: d * scale}


def _check(win, seed, dstate=None, dparams=None, params=None):
    from dynearthsol_gb300.adjoint import adjoint_dot, central_fd
    win.run(params)
    start, grad = win.gradients(seed)
    ad = adjoint_dot(start, grad, dstate, dparams)
    fd = central_fd(win, seed, dstate, dparams, params=params)
    rel = abs(ad - fd) / max(abs(ad), abs(fd), 1e-300)
    return ad, fd, rel


def test_reverse_one_step_start_state():
    """One step, each start-state field alone: adjoint vs central difference."""
    rng = np.random.default_rng(1)
    win = _window(_workload(), 1, 1)
    seed = _seed(win, rng)
    worst = 0.0
    for f in ("coord", "vel", "temperature", "stress", "volume_old"):
        ad, fd, rel = _check(win, seed, dstate=_dstate(win, rng, f))
        print(f"  d{f:12s} adjoint {ad: .9e}  fd {fd: .9e}  rel {rel:.2e}")
        worst = max(worst, rel)
    assert worst <= 1e-6, worst


def test_reverse_one_step_parameters():
    """One step, each parameter alone: shear modulus, cohesion, friction
    angle, conductivity and the prescribed boundary velocities.  The
    conductivity moves only the temperature, by ~1e-12 of the loss: it is
    checked on a temperature seed with a 1e-3 step."""
    from dynearthsol_gb300 import capi
    rng = np.random.default_rng(2)
    wl = _workload()
    ne = wl.mesh.nelem
    wl.elem_fields = {capi.EF_SHEAR_MODULUS: np.full(ne, wl.mat.shear_modulus[0]),
                      capi.EF_COHESION0: np.full(ne, wl.mat.cohesion0[0]),
                      capi.EF_COHESION1: np.full(ne, wl.mat.cohesion1[0]),
                      capi.EF_FRICTION0: np.full(ne, wl.mat.friction_angle0[0]),
                      capi.EF_FRICTION1: np.full(ne, wl.mat.friction_angle1[0]),
                      capi.EF_THERM_COND: np.full(ne, wl.mat.therm_cond[0])}
    win = _window(wl, 1, 1)
    seed = _seed(win, rng)
    worst = 0.0
    for k, base in wl.elem_fields.items():
        if k == capi.EF_THERM_COND:
            continue
        d = rng.standard_normal(ne) * 1e-6 * np.abs(base)
        ad, fd, rel = _check(win, seed, dparams={k: d})
        print(f"  d elem field {k}: adjoint {ad: .9e}  fd {fd: .9e}  rel {rel:.2e}")
        if ad == 0 and fd == 0:
            continue   # no element at yield in this state
        worst = max(worst, rel)
    dv = np.zeros(capi.NBDRY)
    dv[:2] = win.base_vbc[:2] * 1e-6
    ad, fd, rel = _check(win, seed, dparams={"vbc_values": dv})
    print(f"  d vbc_values: adjoint {ad: .9e}  fd {fd: .9e}  rel {rel:.2e}")
    worst = max(worst, rel)
    tseed = {"temperature": seed["temperature"]}
    d = rng.standard_normal(ne) * 1e-3 * wl.mat.therm_cond[0]
    ad, fd, rel = _check(win, tseed, dparams={capi.EF_THERM_COND: d})
    print(f"  d therm_cond: adjoint {ad: .9e}  fd {fd: .9e}  rel {rel:.2e}")
    worst = max(worst, rel)
    assert worst <= 1e-6, worst


def test_reverse_log10_viscosity():
    """Per-element log10 viscosity replacing the viscosity law, 3 steps."""
    from dynearthsol_gb300 import capi
    rng = np.random.default_rng(3)
    wl = _workload()
    ne = wl.mesh.nelem
    wl.elem_fields = {capi.EF_LOG10_VISC: 21 + 0.5 * rng.standard_normal(ne)}
    win = _window(wl, 3, 2)
    seed = _seed(win, rng)
    seed = {"vel": seed["vel"], "stress": seed["stress"]}
    d = rng.standard_normal(ne) * 1e-3
    ad, fd, rel = _check(win, seed, dparams={capi.EF_LOG10_VISC: d})
    print(f"  d log10 visc: adjoint {ad: .9e}  fd {fd: .9e}  rel {rel:.2e}")
    assert rel <= 1e-5, rel


def test_reverse_window_checkpointing_is_exact():
    """The gradients do not depend on the checkpoint spacing (the recompute
    is bit-reproducible): 12 steps checkpointed every 5 (the forward tapes
    the last segment, the backward recomputes the other two) equal 12 steps
    checkpointed every 3 and the window taped whole by its forward
    (checkpoint_every 12, and 100).  A second backward, which finds the
    tape holding the first segment, gives the same bits.  The gradients
    match the central difference."""
    rng = np.random.default_rng(4)
    win = _window(_workload(), 12, 5)
    seed = _seed(win, rng)
    win.run()
    s5, g5 = win.gradients(seed)
    for C in (5, 3, 12, 100):
        win.C = C
        win.run()
        for _ in range(2):
            sC, gC = win.gradients(seed)
            for k in FIELDS:
                np.testing.assert_array_equal(s5[k], sC[k], err_msg=f"{k}, checkpoint_every {C}")
            np.testing.assert_array_equal(g5["vbc_values"], gC["vbc_values"])
            for k, g in g5.items():
                if k != "vbc_values":
                    np.testing.assert_array_equal(g, gC[k], err_msg=f"grad {k}, checkpoint_every {C}")
    win.C = 5
    for f in ("vel", "stress", "coord"):
        ad, fd, rel = _check(win, seed, dstate=_dstate(win, rng, f))
        print(f"  12 steps d{f:8s} adjoint {ad: .9e}  fd {fd: .9e}  rel {rel:.2e}")
        assert rel <= 1e-5, (f, rel)


def _yield_window(rt, K, C):
    from dataclasses import replace
    from cases import build_case
    from dynearthsol_gb300 import capi
    wl, _ = build_case("3d_evp_yield")
    wl.params = replace(wl.params, damping_option=2)
    wl.mat = replace(wl.mat, rheol_type=rt)
    ne = wl.mesh.nelem
    wl.elem_fields = {capi.EF_COHESION1: np.full(ne, wl.mat.cohesion1[0]),
                      capi.EF_FRICTION1: np.full(ne, wl.mat.friction_angle1[0])}
    win = _window(wl, K, C, spin=20)
    final = win.run()
    assert (final["plstrain"] > win.start["plstrain"] + 1e-12).sum() > 0, "no element yields"
    return wl, win


def test_reverse_yielding_elasto_plastic():
    """Mohr-Coulomb return map active (elasto-plastic): start-state
    directions over 3 steps, and the cohesion / friction-angle gradients of
    the yielding elements (their plastic strain is past the softening
    segment, so the saturated values act) over one step.  Over several
    yielding steps the central difference of a parameter has a rounding floor
    of ~1e-11 of the loss (eigen-solver rounding in the yielding elements),
    above the 1e-10 signal of a random parameter direction."""
    from dynearthsol_gb300 import capi
    rng = np.random.default_rng(5)
    rt = capi.RH_ELASTIC | capi.RH_PLASTIC
    wl, win = _yield_window(rt, 3, 2)
    ne = wl.mesh.nelem
    seed = _seed(win, rng)
    for f in ("vel", "stress", "coord"):
        ad, fd, rel = _check(win, seed, dstate=_dstate(win, rng, f))
        print(f"  EP d{f:8s} adjoint {ad: .9e}  fd {fd: .9e}  rel {rel:.2e}")
        assert rel <= 1e-5, (f, rel)
    wl, win = _yield_window(rt, 1, 1)
    seed = _seed(win, rng)
    for k, base in wl.elem_fields.items():
        d = rng.standard_normal(ne) * 1e-6 * np.abs(base)
        ad, fd, rel = _check(win, seed, dparams={k: d})
        print(f"  EP d elem field {k}: adjoint {ad: .9e}  fd {fd: .9e}  rel {rel:.2e}")
        assert ad != 0 and rel <= 1e-5, (k, ad, rel)


@pytest.mark.parametrize("rheology", ["EP", "EVP"])
def test_reverse_yielding_window_is_the_chain_of_one_step_adjoints(rheology):
    """Over 6 yielding steps (checkpoint every 4: one recomputed segment, one
    taped) the window's adjoint equals the chain of six one-step adjoints,
    each from the state the forward reached: the same final state bit for
    bit, the same start-state adjoint and parameter gradients to summation
    order.  The links pass the adjoint of volume_old too: the end state's
    volume_old is the volume at the step's start, which the next step's
    Maxwell update reads (vol / vol_old - 1).  Each link is a one-step
    adjoint, which the one-step tests hold to central differences; over the
    chain itself central differences have a rounding floor above the signal
    (see test_reverse_yielding_elasto_plastic)."""
    from dynearthsol_gb300 import capi
    rng = np.random.default_rng(9)
    rt = capi.RH_ELASTIC | capi.RH_PLASTIC | (capi.RH_VISCOUS if rheology == "EVP" else 0)
    wl, win = _yield_window(rt, 6, 4)
    seed = _seed(win, rng)
    final = win.run()
    s_w, g_w = win.gradients(seed)
    fin_c, s_c, g_c = win.chained_gradients(seed)
    for k in FIELDS:
        np.testing.assert_array_equal(fin_c[k], final[k], err_msg=k)
    assert "volume_old" in s_w
    for k in s_w:
        e = np.abs(s_c[k] - s_w[k]).max() / max(np.abs(s_w[k]).max(), 1e-300)
        assert e <= 1e-12, (k, e)
    yielded = final["plstrain"] > win.start["plstrain"] + 1e-12
    for k, g in g_w.items():
        e = np.abs(g_c[k] - g).max() / max(np.abs(g).max(), 1e-300)
        assert e <= 1e-12, (k, e)
    for k in (capi.EF_COHESION1, capi.EF_FRICTION1):
        assert np.count_nonzero(g_w[k][yielded]) > 0, k
    print(f"  {rheology}: {yielded.sum()} elements yield; chain == window")


def test_reverse_yielding_visco_elasto_plastic_one_step():
    """The EVP branch choice with elements at yield, one step.  Over several
    steps the choice of some elements flips within the finite-difference
    perturbation, which the central difference then straddles."""
    from dynearthsol_gb300 import capi
    rng = np.random.default_rng(6)
    wl, win = _yield_window(capi.RH_ELASTIC | capi.RH_VISCOUS | capi.RH_PLASTIC, 1, 1)
    seed = _seed(win, rng)
    for f in ("vel", "stress", "volume_old"):
        ad, fd, rel = _check(win, seed, dstate=_dstate(win, rng, f))
        print(f"  EVP d{f:8s} adjoint {ad: .9e}  fd {fd: .9e}  rel {rel:.2e}")
        assert rel <= 1e-5, (f, rel)


def test_reverse_matches_fp64_cpu_forward():
    """The gradient of a top-surface velocity misfit with respect to the
    per-element log10 viscosity (8 steps), against fourth-order central
    differences of the CPU FP64 forward -- the oracle, the C restatement of
    the reference -- run from the same start state with dt held (fixed_dt =
    the window's dt).  h = 0.01: below that the differences of the
    quasi-static velocity misfit are dominated by rounding, and a two-point
    difference at that step carries a truncation error of ~3e-4."""
    from dataclasses import replace
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.adjoint import fd5, surface_velocity_misfit, top_nodes
    from oracle.oracle import Oracle, state_copy
    rng = np.random.default_rng(8)
    LV = capi.EF_LOG10_VISC
    wl = _workload()
    ne = wl.mesh.nelem
    lv_t = 21 + 0.5 * rng.standard_normal(ne)
    lv_s = 21 + 0.5 * rng.standard_normal(ne)
    wl.elem_fields = {LV: lv_s}
    K = 8
    win = _window(wl, K, 4)
    nodes = top_nodes(wl.mesh)
    target = win.run({LV: lv_t})["vel"]
    final = win.run({LV: lv_s})
    loss, seed = surface_velocity_misfit(final["vel"], target, nodes)
    _, g = win.gradients({"vel": seed})
    g = g[LV]
    win.m.upload(win.start, win.clock)
    full = win.m.download()   # the start state with its derived fields
    wl_cpu = replace(wl, params=replace(wl.params, fixed_dt=win.clock[1]))

    def cpu_loss(lv):
        st = state_copy(full)
        wl_cpu.elem_fields = {LV: lv}
        o = Oracle(wl_cpu, st, win.m.comp_pressure, 1, win.clock)
        assert o.run(K) == 0
        return surface_velocity_misfit(st["vel"], target, nodes)[0]

    assert abs(cpu_loss(lv_s) - loss) <= 1e-9 * loss   # the two forwards agree
    worst = 0.0
    for e in np.argsort(-np.abs(g))[:6]:
        def along(t, e=e):
            lv = lv_s.copy()
            lv[e] += t
            return cpu_loss(lv)
        fd = fd5(along, 1e-2)
        rel = abs(fd - g[e]) / max(abs(fd), abs(g[e]))
        print(f"  elem {e:4d}: adjoint {g[e]: .9e}  cpu fd {fd: .9e}  rel {rel:.2e}")
        worst = max(worst, rel)
    assert worst <= 1e-4, worst


def test_reverse_torch_autograd_function():
    """The torch.autograd.Function wrapper: a misfit built in torch from the
    window's final velocities, loss.backward() through the adjoint; its
    gradients equal the adjoint's and match a central difference."""
    torch = pytest.importorskip("torch")
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.adjoint import fd5, top_nodes, window_function
    rng = np.random.default_rng(9)
    wl = _workload()
    ne = wl.mesh.nelem
    lv0 = 21 + 0.5 * rng.standard_normal(ne)
    wl.elem_fields = {capi.EF_LOG10_VISC: lv0, capi.EF_SHEAR_MODULUS: np.full(ne, wl.mat.shear_modulus[0])}
    win = _window(wl, 6, 3)
    WF = window_function()
    nodes = torch.from_numpy(top_nodes(wl.mesh))
    target = torch.from_numpy(win.run({capi.EF_LOG10_VISC: lv0 + 0.3})["vel"])

    def loss_fn(lv, G):
        v = WF.apply(win, lv, G, None, None, None, None, None, None)
        return 0.5 * ((v[nodes] - target[nodes]) ** 2).sum()

    lv = torch.tensor(lv0, dtype=torch.float64, requires_grad=True)
    G = torch.tensor(wl.elem_fields[capi.EF_SHEAR_MODULUS], dtype=torch.float64, requires_grad=True)
    loss = loss_fn(lv, G)
    loss.backward()
    d_lv = rng.standard_normal(ne) * 1e-2
    d_G = rng.standard_normal(ne) * 1e-3 * float(wl.mat.shear_modulus[0])
    ad = float(lv.grad.numpy() @ d_lv + G.grad.numpy() @ d_G)
    with torch.no_grad():
        fd = fd5(lambda t: float(loss_fn(torch.from_numpy(lv0 + t * d_lv),
                                         torch.from_numpy(G.detach().numpy() + t * d_G))), 1.0)
    rel = abs(fd - ad) / max(abs(fd), abs(ad))
    print(f"  autograd: adjoint {ad: .9e}  fd {fd: .9e}  rel {rel:.2e}")
    assert rel <= 1e-5, rel


def test_window_tape_too_large_is_enomem_and_context_survives():
    """A window whose tape cannot fit on the device (1000 steps of the
    998,400-tet case, ~367 GB) is refused with DES_ENOMEM before any
    allocation, and the context keeps working: the next upload and step run
    and leave no device error."""
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import initial_state, make_workload
    from dynearthsol_gb300.solver import DeviceModel
    wl = make_workload("c1_3d_evp")
    st, cp = initial_state(wl)
    m = DeviceModel(wl, comp_pressure=cp)
    init = m.init_fields(st)
    clk = m.clock()
    with pytest.raises(capi.DesError) as ex:
        m.adjoint_forward(1000, 1000)
    assert ex.value.code == capi.DES_ENOMEM, ex.value
    m.upload(init, clk)
    m.step(2)
    m.sync()
    assert m.device_status() == 0
    assert np.isfinite(m.download()["vel"]).all()
    m.close()

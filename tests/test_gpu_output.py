"""des_write_save: an output frame written from device buffers, in the
reference's .save layout (the layout itself is pinned against the
reference's BinaryOutput in test_save_format.py).  The state arrays must
equal the downloaded state; the per-element density, viscosity, mesh quality
and material are checked against restatements of MatProps::rho/visc
(matprops.cxx:276-312,376-397), elem_quality's minimum
(des_worst_elem_quality) and the most abundant marker."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rho_visc(wl, st):
    """MatProps::rho and ::visc with marker blending, from a host state."""
    m, mt = wl.mesh, wl.mat
    nd, ne = m.ndims, m.nelem
    conn = m.connectivity
    T = st["temperature"][conn].sum(axis=1) / (nd + 1)
    em = mt.elemmarkers if mt.elemmarkers is not None else np.ones((ne, 1), dtype=np.int64)
    nmat = em.shape[1]
    n = em.sum(axis=1)
    rho = sum(mt.rho0[k] * (1 - mt.alpha[k] * (T - 273)) * em[:, k] for k in range(nmat)) / n
    s = st["strain_rate"]
    if nd == 3:
        a = s[:, :3].sum(axis=1) / 3
        j2 = 0.5 * ((s[:, 0] - a) ** 2 + (s[:, 1] - a) ** 2 + (s[:, 2] - a) ** 2) + (s[:, 3:] ** 2).sum(axis=1)
    else:
        j2 = 0.25 * (s[:, 0] - s[:, 1]) ** 2 + s[:, 2] ** 2
    ed = np.maximum(np.sqrt(j2), 1e-30)
    acc = 0.0
    for k in range(nmat):
        nexp = mt.visc_exponent[k]
        v0 = (0.25 * ed ** (1 / nexp - 1) * (0.75 * mt.visc_coefficient[k]) ** (-1 / nexp)
              * np.exp(mt.visc_activation_energy[k] / (nexp * 8.3144 * T)) * 1e6)
        acc = acc + em[:, k] / v0
    visc = np.clip(n / acc, mt.visc_min, mt.visc_max)
    mat = np.argmax(em, axis=1).astype(np.float64)
    return rho, visc, mat


@pytest.mark.parametrize("case", ["3d_heat_jitter_multimat", "3d_evp_yield", "2d_evp_heat"])
def test_write_save_from_device(case, tmp_path):
    import ctypes as C
    from cases import build_case
    from dynearthsol_gb300 import capi
    from dynearthsol_gb300.config import initial_state
    from dynearthsol_gb300.solver import DeviceModel
    wl, _ = build_case(case)
    st, cp = initial_state(wl)
    m = DeviceModel(wl, comp_pressure=cp)
    m.init_fields(st)
    m.step(15)
    path = tmp_path / f"{case}.save.000000"
    assert m.lib.des_write_save(m.ctx, str(path).encode()) == 0
    s = m.download()
    f = capi.read_save(str(path))
    assert f["ndims"] == wl.mesh.ndims
    exact = {"coordinate": "coord", "velocity": "vel", "temperature": "temperature",
             "plastic strain": "plstrain", "plastic strain-rate": "delta_plstrain", "strain-rate": "strain_rate",
             "strain": "strain", "stress": "stress", "force": "force", "coord0": "coord0"}
    for name, key in exact.items():
        np.testing.assert_array_equal(f[name], s[key].ravel(), err_msg=name)
    np.testing.assert_array_equal(f["connectivity"], wl.mesh.connectivity.ravel())
    np.testing.assert_array_equal(f["bcflag"], wl.mesh.bcflag)
    rho, visc, mat = _rho_visc(wl, s)
    np.testing.assert_allclose(f["density"], rho, rtol=1e-13)
    np.testing.assert_allclose(f["viscosity"], visc, rtol=1e-11)
    np.testing.assert_array_equal(f["material"], mat)
    q, w = C.c_double(), C.c_int()
    assert m.lib.des_worst_elem_quality(m.ctx, C.byref(q), C.byref(w)) == 0
    assert f["mesh quality"].min() == q.value and int(np.argmin(f["mesh quality"])) == w.value
    assert np.all(f["mesh quality"] > 0) and np.all(f["mesh quality"] <= 1 + 1e-12)
    m.close()

"""Generate the golden fixtures of tests/golden/ from the REFERENCE itself.

Runs only where the reference tree exists (it compiles the reference's own
fields/geometry/rheology/matprops/bc/ic sources and 3x3-C through
``make -C oracle ref`` and drives them with oracle/ref_harness.cxx).  For
every case of tests/cases.py it stores, bit for bit:

* ``init/*``  -- the state after the reference's init sequence
  (dynearthsol.cxx:82-98: volumes, masses, shape functions, boundary
  normals, velocity BCs, initial stress, weak zone, dt);
* ``final/*`` -- the state after ``nsteps`` of the loop body
  (dynearthsol.cxx:325-361) and the dt of every step;
* for the per-function cases, ``mid/*`` (the state after 60 steps, or
  ``cases.MID_STEPS``),
  ``fn_<name>/*`` -- the fields each reference function writes when applied
  once to ``mid`` (plus compute_dt and worst_elem_quality results) -- and
  ``mid1/*``, ``mid10/*``: the state 1 and 10 steps after ``mid``, with
  their envelopes ``envelope_mid1/*``, ``envelope_mid10/*`` (below);
  the full-horizon cases keep fewer fields (``kept``) and no ``fn_*``;
* ``envelope/<field>`` -- the libm sensitivity of the case: the largest
  normalised deviation from ``final`` of three runs of the restatement whose
  transcendental results are moved by +-1 ulp (seeds 1, 2, 3).  Any faithful
  FP64 implementation with a different libm lands inside a small multiple of
  it; plastic 3D cases are chaotic enough that it exceeds 1e-9.

Usage:  python tests/golden/gen_golden.py [case ...]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from dataclasses import replace  # noqa: E402

from cases import (CASES, FULL_CASES, FUNCTIONS, PERFN_CASES, build_case, mid_steps,  # noqa: E402
                   reference_material_for)
from dynearthsol_gb300.config import initial_state  # noqa: E402
from oracle.oracle import Oracle, Reference, build_reference, state_copy  # noqa: E402

ENVELOPE_FIELDS = ("vel", "stress", "temperature", "plstrain", "coord", "strain", "force", "delta_plstrain")
# the full-horizon cases are large (up to 14,400 tets): their final and
# mid+k states keep the compared fields only (fewer in 3D), and they keep no
# per-function outputs (the one-step run from mid checks every function)
LEAN_FIELDS_2D = ENVELOPE_FIELDS + ("volume", "dpressure", "delta_plstrain")
LEAN_FIELDS_3D = ("vel", "stress", "temperature", "plstrain", "coord", "delta_plstrain")


def kept(name: str, k: str) -> bool:
    if name not in FULL_CASES:
        return True
    return k in (LEAN_FIELDS_2D if name.startswith("2d") else LEAN_FIELDS_3D)


def envelope(wl, start, cp, clk, nsteps, result):
    """Largest normalised deviation from ``result`` over three runs of the
    restatement with +-1 ulp perturbed transcendentals (seeds 1, 2, 3)."""
    env = {f: 0.0 for f in ENVELOPE_FIELDS}
    for seed in (1, 2, 3):
        s = state_copy(start)
        o = Oracle(wl, s, cp, 1, (clk[0], clk[1], int(clk[2])), perturb_seed=seed)
        assert o.run(nsteps) == 0
        for f in ENVELOPE_FIELDS:
            scale = np.abs(result[f]).max()
            d = np.abs(s[f] - result[f]).max()
            env[f] = max(env[f], float(d / scale) if scale else float(d))
        del o
    return env


def gen(name: str) -> str:
    wl, nsteps = build_case(name)
    wl_ref = replace(wl, mat=reference_material_for(wl), elem_fields={})
    ref = Reference(wl.mesh.ndims)
    st, comp = initial_state(wl)
    out = {}
    bn, ev, cp, clk = ref.init(wl_ref, st)
    for k, v in st.items():
        out[f"init/{k}"] = v.copy()
    out["init/bnormals"] = bn
    out["init/edge_vectors"] = ev
    out["init/clock"] = np.array(clk, dtype=np.float64)
    out["init/compensation_pressure"] = np.array(cp)
    if name in PERFN_CASES:
        mid = state_copy(st)
        clk_mid, _ = ref.run(wl_ref, mid, cp, clk, mid_steps(name))
        for k, v in mid.items():
            out[f"mid/{k}"] = v.copy()
        out["mid/clock"] = np.array(clk_mid, dtype=np.float64)
        for fn, fields in FUNCTIONS.items():
            if name in FULL_CASES:
                continue
            s = state_copy(mid)
            ref.call(wl_ref, s, cp, clk_mid, fn)
            for f in fields:
                out[f"fn_{fn}/{f}"] = s[f].copy()
        for k_steps in (1, 10):
            s = state_copy(mid)
            clk_k, _ = ref.run(wl_ref, s, cp, clk_mid, k_steps)
            for k, v in s.items():
                if kept(name, k):
                    out[f"mid{k_steps}/{k}"] = v.copy()
            out[f"mid{k_steps}/clock"] = np.array(clk_k, dtype=np.float64)
            for f, v in envelope(wl, mid, cp, clk_mid, k_steps, s).items():
                out[f"envelope_mid{k_steps}/{f}"] = np.array(v)
        s = state_copy(mid)
        res, _ = ref.call(wl_ref, s, cp, clk_mid, "compute_dt")
        out["fn_compute_dt/dt"] = np.array(res[0])
        s = state_copy(mid)
        res, _ = ref.call(wl_ref, s, cp, clk_mid, "worst_elem_quality")
        out["fn_worst_elem_quality/result"] = res.copy()
    init_state = state_copy(st)
    clk_f, dts = ref.run(wl_ref, st, cp, clk, nsteps)
    for k, v in st.items():
        if kept(name, k):
            out[f"final/{k}"] = v.copy()
    for f, v in envelope(wl, init_state, cp, clk, nsteps, st).items():
        out[f"envelope/{f}"] = np.array(v)
    out["final/clock"] = np.array(clk_f, dtype=np.float64)
    out["final/dts"] = dts
    out["nsteps"] = np.array(nsteps)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    return path


def main(argv):
    if not build_reference():
        print("reference tree not found; cannot generate fixtures", file=sys.stderr)
        return 1
    names = argv or CASES
    for n in names:
        p = gen(n)
        print(f"{n}: {os.path.getsize(p) / 1024:.1f} KiB")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))

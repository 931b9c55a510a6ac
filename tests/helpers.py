"""Shared helpers of the test-suite: build the same experiment on the GPU (through the
package API) and in the CPU oracle, with the same seeded initial state."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

PROG = ["b", "u_i", "u_j", "u_k"]
DIAG = ["p", "ke", "U_i", "U_j", "U_k", "vor_i", "vor_j", "vor_k", "div"]


def make_params(geometry="closed", modelname="LES", timestepping="RK3_SSP", n=(16, 8, 8), L=(1.0, 1.0, 1.0),
                n_tracers=0, auto_dt=False, dt=1e-3, cfl=0.8, dt_max=1.0, rotating=False, coriolis=1.0,
                diff_coef=None, precision="fp64", mg_tol=1e-6, mg_maxite=20, forced=False, tracer_diffusion=False,
                tracer_scheme="weno", orderA=5, vf_scheme="weno", orderVF=5):
    from nyles_gb300 import parameters
    parameters.InextensibleDict.unfreeze()
    p = parameters.UserParameters()
    p.model["modelname"] = modelname
    p.model["geometry"] = geometry
    p.model["Lx"], p.model["Ly"], p.model["Lz"] = L
    p.model["n_tracers"] = n_tracers
    p.time["timestepping"] = timestepping
    p.time["auto_dt"] = auto_dt
    p.time["dt"] = dt
    p.time["cfl"] = cfl
    p.time["dt_max"] = dt_max
    p.physics["rotating"] = rotating
    p.physics["coriolis"] = coriolis
    p.physics["diff_coef"] = dict(diff_coef or {})
    p.physics["forced"] = forced
    p.discretization["global_nx"], p.discretization["global_ny"], p.discretization["global_nz"] = n
    p.gpu["precision"] = precision
    p.gpu["mg_tol"] = mg_tol
    p.gpu["mg_maxite"] = mg_maxite
    p.gpu["history"] = False
    p.gpu["tracer_diffusion"] = tracer_diffusion
    p.gpu["tracer_scheme"] = tracer_scheme
    p.discretization["orderA"] = orderA
    p.gpu["vf_scheme"] = vf_scheme
    p.discretization["orderVF"] = orderVF
    return p


def oracle_for(nyl):
    """OracleModel with the same descriptor as a GPU Nyles instance."""
    import oracle
    prm = nyl.param
    g = nyl.grid
    m = nyl.model
    visc = prm["diff_coef"].get("u") if prm["diff_coef"] else None
    live = prm["gpu"].get("tracer_diffusion") or prm["modelname"] == "advection"
    trd = {k: v for k, v in prm["diff_coef"].items() if k != "u"} if live and prm["diff_coef"] else None
    order = prm["orderA"] if prm["gpu"].get("tracer_scheme") == "linear" else 0
    vf_order = prm["orderVF"] if prm["gpu"].get("vf_scheme") == "linear" else 0
    o = oracle.OracleModel(dict(nx=prm["nx"], ny=prm["ny"], nz=prm["nz"], nh=prm["nh"], geometry=prm["geometry"],
                                n_tracers=prm["n_tracers"], modelname=prm["modelname"],
                                timestepping=prm["timestepping"], dx=g.dx, dy=g.dy, dz=g.dz, idx2=g.idx2,
                                idy2=g.idy2, idz2=g.idz2, fparam=float(m.fparameter), visc=visc,
                                tracer_diffusion=trd, tracer_order=order, vf_order=vf_order))
    o.mg_params(prm["gpu"]["mg_tol"], prm["gpu"]["mg_maxite"], prm["gpu"]["mg_omega"])
    return o


def seeded_state(nyl, kind, seed):
    """Initial fields (numpy, (z, y, x)) written through view('i'), walls at rest."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g = nyl.grid
    st = nyl.model.state
    shape = tuple(st.b.view("i").shape)
    out = {k: np.zeros(shape) for k in PROG}
    for t in range(nyl.param["n_tracers"]):
        out["t%d" % t] = np.zeros(shape)
    xb, zb = g.x_b.view("i").numpy(), g.z_b.view("i").numpy()
    if kind == "lock":
        out["b"] = np.where(xb < 0.5 * g.Lx, -0.5, 0.5) + 1e-3 * rng.uniform(-1, 1, size=shape)
    elif kind == "noise":
        out["b"] = zb + 1e-2 * rng.standard_normal(shape)
        for k, d in zip(["u_i", "u_j", "u_k"], [g.dx, g.dy, g.dz]):
            out[k] = 1e-1 * rng.standard_normal(shape) * d
        for t in range(nyl.param["n_tracers"]):
            out["t%d" % t] = np.tanh((zb - 0.5 * g.Lz) / (0.1 * g.Lz)) + 1e-2 * rng.standard_normal(shape)
    elif kind == "tgv":
        xu, yu, zu = (g.x_vel["i"].view("i").numpy(), g.y_vel["i"].view("i").numpy(), g.z_vel["i"].view("i").numpy())
        xv, yv, zv = (g.x_vel["j"].view("i").numpy(), g.y_vel["j"].view("i").numpy(), g.z_vel["j"].view("i").numpy())
        out["u_i"] = (np.sin(xu) * np.cos(yu) * np.cos(zu) + 1e-4 * rng.standard_normal(shape)) * g.dx
        out["u_j"] = (-np.cos(xv) * np.sin(yv) * np.cos(zv) + 1e-4 * rng.standard_normal(shape)) * g.dy
        out["u_k"] = 1e-4 * rng.standard_normal(shape) * g.dz
    geo = nyl.param["geometry"]
    if "x" not in geo:
        out["u_i"][:, :, -1] = 0.0
    if "y" not in geo:
        out["u_j"][:, -1, :] = 0.0
    if "z" not in geo:
        out["u_k"][-1, :, :] = 0.0
    return out


def load_state(nyl, o, fields):
    import torch
    for k, v in fields.items():
        nyl.model.state.get(k).view("i")[...] = torch.from_numpy(v)
        o.field(k)[...] = v


def relerr(a, b, scale=None):
    """max|a-b| / max|b| (or / scale)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.max(np.abs(b)) if scale is None else scale, 1e-300)
    return float(np.max(np.abs(a - b)) / den)


VECTORS = {"u": ("u_i", "u_j", "u_k"), "U": ("U_i", "U_j", "U_k"), "vor": ("vor_i", "vor_j", "vor_k")}


def parity_errors(get_a, get_b, names):
    """Relative max-norm error per variable. Scalars are normalised by their own
    max-norm; components of a vector field (u, U, vor) by the max-norm of the whole
    vector, so that a component that is only round-off noise (v in a 2-D flow) is
    measured against the velocity scale, not against its own noise level."""
    out = {}
    scales = {}
    for vec, comps in VECTORS.items():
        if any(c in names for c in comps):
            scales[vec] = max(float(np.max(np.abs(np.asarray(get_b(c), dtype=np.float64)))) for c in comps)
    for n in names:
        vec = next((v for v, comps in VECTORS.items() if n in comps), None)
        out[n] = relerr(get_a(n), get_b(n), scales.get(vec))
    return out


def golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    return d, meta

"""The learned correction: quiescent-gas training runs, features, training and
evaluation, all on the GPU through the library (pstep, pgas, pmlp).

Training data. Isolated particles move through gas at rest (u = 0, rho = T = 1)
with the two-way-coupled step: the FP32 particle step deposits its drag and
heat into the box gas step (grid.cpp), whose response disturbs the gas at each
particle. The undisturbed state is known (u = 0, T = 1), so the gas values the
plain interpolation gives at a particle are exactly its self-induced
disturbance. Each particle has d_p/dx ~ U[0.05, 1], Re_p ~ logU[0.1, 50],
heating Q ~ U[0, 2] and a slip of uniform random direction; a body force equal
to m_p slip / tau_p holds that slip as its terminal velocity, and the particle
starts at it and at its steady excess temperature Q tau_T (tau_T = 0.15, the
thermal response time of the box workloads, so the excess stays below 0.3).
Particles sit in random positions inside the cells of a lattice of spacing
16 dx (8^3 = 512 per 128^3 box), so each is isolated; 8 boxes give 4096.

The ratio Re_p / (d_p/dx) = |slip| dx / nu sets how fast a particle crosses a
cell relative to viscous diffusion over one. Particles are grouped into the 8
boxes by it, and each box's gas viscosity is chosen so that its fastest
particle moves at most 0.05 cells per step and viscous diffusion stays at or
below 0.05 dx^2 per step: every particle then either out-runs or out-diffuses
its own wake within a few tens of steps, and the disturbance is quasi-steady
when recording starts (step 100 of 200).

Targets and features. The network predicts the disturbance in units of the
particle's current slip s = u_p - u_gas and excess temperature T_p - Tg:
  y = (u_gas / |s|, (Tg - 1) / (T_p - Tg))
from features (offset of the particle in its cell, s/|s|, d_p/dx, ln Re_p with
Re_p = |s| d_p / nu, Q, ln tau_p), normalised to about [-1, 1] by fixed
affine maps stored with the model. The step applies it as documented in
pstep.h (pstep_correction).
"""
from __future__ import annotations

import dataclasses
import json
import math
import os

import numpy as np

from . import gas, mlp, pstep
from .config import PI

FEATURES = ["ox", "oy", "oz", "sx", "sy", "sz", "dp_dx", "ln_re_p", "q", "ln_tau_p"]
# The disturbance per unit drive slip follows (d_p/dx) / (1 + Re_cell / PRIOR_RE), Re_cell = Re_p/(d_p/dx),
# over the whole training range (fitted to the plain runs); the network learns the O(1) remainder.
PRIOR_RE = 3.3
TARGET_CLIP = 10.0
MODEL_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "correction_quiescent.npz")


@dataclasses.dataclass
class Spec:
    n: int = 128
    runs: int = 8
    lattice: int = 16
    steps: int = 200
    record_from: int = 100
    dt: float = 1e-3
    l: float = 2 * PI
    rho_ratio: float = 1000.0
    prandtl: float = 0.7
    nusselt: float = 2.0
    cp: float = 3.5
    cv: float = 2.5
    cfl_max: float = 0.05
    visc_max: float = 0.05
    dp_range: tuple = (0.05, 1.0)
    re_range: tuple = (0.1, 50.0)
    q_range: tuple = (0.0, 2.0)
    tau_t: float = 0.15

    @property
    def dx(self) -> float:
        return self.l / self.n

    @property
    def per_run(self) -> int:
        return (self.n // self.lattice) ** 3


def sample(spec: Spec, seed: int) -> list[dict]:
    """Particles of all boxes: per box the particle parameters, lattice positions and gas viscosity."""
    rng = np.random.default_rng(seed)
    m = spec.runs * spec.per_run
    dp_dx = rng.uniform(*spec.dp_range, m)
    re_p = np.exp(rng.uniform(math.log(spec.re_range[0]), math.log(spec.re_range[1]), m))
    q = rng.uniform(*spec.q_range, m)
    d = rng.normal(size=(m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    order = np.argsort(re_p / dp_dx, kind="stable")
    side = spec.n // spec.lattice
    runs = []
    for r in range(spec.runs):
        idx = order[r * spec.per_run:(r + 1) * spec.per_run]
        re_cell = re_p[idx] / dp_dx[idx]  # |slip| dx / nu
        # viscosity: fastest particle at cfl_max cells per step, diffusion number <= visc_max
        visc = min(spec.visc_max, spec.cfl_max / float(re_cell.max()))
        nu = visc * spec.dx ** 2 / spec.dt
        a, b, c = np.meshgrid(np.arange(side), np.arange(side), np.arange(side), indexing="ij")
        sites = np.stack([a.ravel(), b.ravel(), c.ravel()], axis=1) * spec.lattice + spec.lattice // 2
        pos = (sites + rng.uniform(0.0, 1.0, (spec.per_run, 3))) * spec.dx
        runs.append(dict(dp_dx=dp_dx[idx], re_p=re_p[idx], q=q[idx], dir=d[idx], pos=pos, nu=nu))
    return runs


def _box(spec: Spec, run: dict):
    """Gas and particle-step configurations and per-particle properties of one box."""
    nu = run["nu"]
    k_gas = spec.cp * nu / spec.prandtl  # thermal diffusivity nu / Pr with rho0 = 1
    dx = spec.dx
    dp = run["dp_dx"] * dx
    mp = spec.rho_ratio * PI * dp ** 3 / 6.0
    tau_p = spec.rho_ratio * dp ** 2 / (18.0 * nu)
    itth = spec.nusselt * PI * dp * k_gas
    tau_t = np.full_like(tau_p, spec.tau_t)
    heat_is = 1.0 / (tau_t * itth)  # 1/(m_p Cvp) with tau_T = m_p Cvp / itth
    alpha = run["q"] / heat_is      # heating rate Q = alpha / (m_p Cvp)
    slip = (run["re_p"] * nu / dp)[:, None] * run["dir"]
    accel = slip / tau_p[:, None]
    gcfg = dict(n=spec.n, l=spec.l, dt=spec.dt, mu0=nu, k=k_gas, cp=spec.cp, cv=spec.cv, rho0=1.0, u0=0.0,
                a_force=0.0, gx=0.0, gy=0.0, gz=0.0, mp=1.0, epsilon=1e-10, iterations=30, cooling=1, twc=1, p0=1.0)
    scfg = dict(n=spec.n, l=spec.l, dt=spec.dt, tp=1.0, mp=1.0, dp=float(np.mean(dp)), nu=spec.nusselt, k=k_gas,
                epsilonp=1.0, i0=0.0, cvp=1.0, gx=0.0, gy=0.0, gz=0.0, particle_gravity=0, twc=1)
    props = dict(tau_p=tau_p, mass_ratio=mp, itth=itth, heat_is=heat_is, alpha=alpha,
                 accel=[np.ascontiguousarray(accel[:, i]) for i in range(3)])
    state = dict(x=run["pos"][:, 0].copy(), y=run["pos"][:, 1].copy(), z=run["pos"][:, 2].copy(),
                 u=slip[:, 0].copy(), v=slip[:, 1].copy(), w=slip[:, 2].copy(), t=1.0 + run["q"] * tau_t,
                 flag=np.arange(len(dp), dtype=np.int32))
    return gcfg, scfg, props, state, dict(dp=dp, tau_p=tau_p, q=run["q"], slip0=slip, nu=nu)


def _face_interp(spec: Spec, g, pos: np.ndarray) -> np.ndarray:
    """The plain gas velocity at the particles from the gas fields at the start of a step:
    U = RU / Rho_face (grid.cpp:662, Rho_face = Rho interpolated to faces) interpolated as
    gas2part_velocity (particle.cpp:340-360), in fp64."""
    rho = g.field("Rho")
    idx = spec.n / spec.l
    out = np.empty((len(pos), 3))
    for a, name in enumerate(("RU_x", "RU_y", "RU_z")):
        ru = g.field(name)
        face = 0.5 * (rho + np.roll(rho, 1, axis=2 - a))
        u = ru / face
        c = np.floor(pos * idx).astype(np.int64)
        frac = pos[:, a] * idx - c[:, a]
        i, j, k = c[:, 0] + 1, c[:, 1] + 1, c[:, 2] + 1
        hi = [i, j, k]
        hi[a] = hi[a] + 1
        out[:, a] = frac * u[hi[2], hi[1], hi[0]] + (1 - frac) * u[k, j, i]
    return out


def _temp_interp(spec: Spec, g, pos: np.ndarray) -> np.ndarray:
    """The plain gas temperature at the particles (gas2part_Temp_new, particle.cpp:430-456), fp64."""
    T = g.field("T")
    idx = spec.n / spec.l
    r = np.floor(pos * idx + 0.5).astype(np.int64)
    w = pos * idx - r + 0.5
    ni, nj, nk = r[:, 0] + 1, r[:, 1] + 1, r[:, 2] + 1
    tx, ty, tz = w[:, 0], w[:, 1], w[:, 2]
    return (tx * ty * tz * T[nk, nj, ni] + (1 - tx) * ty * tz * T[nk, nj, ni - 1] + tx * (1 - ty) * tz * T[nk, nj - 1, ni] +
            tx * ty * (1 - tz) * T[nk - 1, nj, ni] + (1 - tx) * (1 - ty) * tz * T[nk, nj - 1, ni - 1] +
            (1 - tx) * ty * (1 - tz) * T[nk - 1, nj, ni - 1] + tx * (1 - ty) * (1 - tz) * T[nk - 1, nj - 1, ni] +
            (1 - tx) * (1 - ty) * (1 - tz) * T[nk - 1, nj - 1, ni - 1])


def run_box(spec: Spec, run: dict, model: dict | None = None, record: bool = True, every_stage: bool = False) -> dict:
    """One quiescent box on the GPU; records, from step record_from on, the state at the start of
    each step and, for stage 0 (x_int = x), the gas values the particle update used (the kept
    values) and the plain interpolation -- the true disturbance. Without a model the two agree;
    with one, the plain values are interpolated here from the gas fields."""
    gcfg, scfg, props, st, const = _box(spec, run)
    count = len(st["flag"])
    ps = pstep.ParticleStep(scfg, count, pstep.FP32, pstep.KEEP_GAS)
    ps.load(*[np.ascontiguousarray(st[k]) for k in ("x", "y", "z", "u", "v", "w", "t", "flag")])
    ps.set_props(**props)
    if model is not None:
        ps.set_correction(model, const["nu"], every_stage=every_stage)
    g = gas.GasStep(gcfg, ps)
    z = np.zeros((spec.n,) * 3)
    g.init(z, z, z, np.ones((spec.n,) * 3), 1.0)
    keys = ("x", "y", "z", "u", "v", "w", "ug", "vg", "wg", "Tg", "T_int", "flag", "up", "vp", "wp", "Tp")
    rec = {k: [] for k in keys}
    for s in range(spec.steps):
        on = record and s >= spec.record_from
        if on:
            base = {k: ps.array(k) for k in ("x", "y", "z", "u", "v", "w", "flag")}
            if model is not None:
                plain_u = _face_interp(spec, g, np.stack([base["x"], base["y"], base["z"]], axis=1))
        g.stage(0)
        if on:
            kept = {k: ps.array(k) for k in ("ug", "vg", "wg", "Tg", "T_int")}
            if model is not None:
                xn = np.stack([ps.array(k) for k in ("x_int", "y_int", "z_int")], axis=1)  # stage 0's x_new
                plain_t = _temp_interp(spec, g, xn)
            else:
                plain_u = np.stack([kept["ug"], kept["vg"], kept["wg"]], axis=1)
                plain_t = kept["Tg"]
            for k in ("x", "y", "z", "u", "v", "w", "flag"):
                rec[k].append(base[k])
            for k in ("ug", "vg", "wg", "Tg", "T_int"):
                rec[k].append(kept[k])
            for a, k in enumerate(("up", "vp", "wp")):
                rec[k].append(plain_u[:, a])
            rec["Tp"].append(plain_t)
        for k in (1, 2, 3):
            g.stage(k)
        g.end_step()
    final = {k: ps.array(k) for k in ("u", "v", "w", "flag")}
    rc, flags = ps.check()
    g.close()
    ps.close()
    if rc != 0 or not all(np.all(np.isfinite(v)) for v in rec["ug"]):
        raise FloatingPointError(f"quiescent box with nu={run['nu']:.3e} left a non-finite state (status {rc})")
    out = {k: np.concatenate(v) if v else np.zeros(0) for k, v in rec.items()}
    out["flag"] = out["flag"].astype(np.int64)
    out["final"] = final
    out["const"] = const
    return out


def raw_features(spec: Spec, rec: dict) -> tuple[np.ndarray, np.ndarray, dict]:
    """(raw features, targets, extras) of recorded samples; per-particle constants by id.

    Features as the kernel forms them: the direction and Re_p of the slip that drove the drag
    (u_p minus the gas velocity the step used; the plain slip in the plain runs).
    Targets: the true disturbance (plain interpolation; the undisturbed state is u = 0,
    T = 1) per unit of that drive slip and drive temperature difference."""
    c = rec["const"]
    idx = 1.0 / spec.dx
    fl = rec["flag"]
    off = np.stack([rec[k] * idx - np.floor(rec[k] * idx) for k in ("x", "y", "z")], axis=1)
    up = np.stack([rec["u"], rec["v"], rec["w"]], axis=1)
    plain = np.stack([rec["up"], rec["vp"], rec["wp"]], axis=1)
    used = np.stack([rec["ug"], rec["vg"], rec["wg"]], axis=1)
    s = up - plain
    smag = np.linalg.norm(s, axis=1)
    sd = up - used
    sdrv = np.linalg.norm(sd, axis=1)
    dp = c["dp"][fl]
    re = sdrv * dp / c["nu"]
    tau = c["tau_p"][fl]
    q = c["q"][fl]
    with np.errstate(divide="ignore", invalid="ignore"):
        f = np.column_stack([off, sd / sdrv[:, None], dp * idx, np.log(re), q, np.log(tau)])
        y_vel = plain / sdrv[:, None]
        tdrv = rec["T_int"] - rec["Tg"]
        y_t = np.where(np.abs(tdrv) > 0, (rec["Tp"] - 1.0) / tdrv, 0.0)
    y = np.column_stack([y_vel, y_t])
    ok = (smag > 0) & (sdrv > 0) & np.all(np.isfinite(f), axis=1) & np.all(np.isfinite(y), axis=1)
    return f[ok], y[ok], dict(smag=smag[ok], slip0=np.linalg.norm(c["slip0"][fl], axis=1)[ok], re=re[ok],
                               tau=tau[ok], q=q[ok], dp_dx=(dp * idx)[ok], gas=used[ok])


def normaliser(f: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """Fixed affine maps to about [-1, 1] (offsets and directions keep their natural scale),
    and the ranges of d_p/dx, Re_p, Q, tau_p seen in training."""
    lo, hi = f.min(axis=0), f.max(axis=0)
    shift = (lo + hi) / 2
    scale = 2.0 / np.maximum(hi - lo, 1e-6)
    shift[:3], scale[:3] = 0.5, 2.0      # offsets in [0, 1)
    shift[3:6], scale[3:6] = 0.0, 1.0    # unit slip direction
    rng_lo = np.array([lo[6], math.exp(lo[7]), lo[8], math.exp(lo[9])])
    rng_hi = np.array([hi[6], math.exp(hi[7]), hi[8], math.exp(hi[9])])
    return shift, scale, rng_lo, rng_hi


def prior(f: np.ndarray) -> np.ndarray:
    """The kernel's output scale for raw features f (pstep_correction.prior_re)."""
    dpdx = f[:, 6]
    return dpdx / (1.0 + np.exp(f[:, 7]) / dpdx / PRIOR_RE)


_PERMS = np.array([(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)])


def symmetry_images(f: np.ndarray, y: np.ndarray, copies: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """The samples and `copies` images of each under random elements of the cube's symmetry
    group (48: axis permutations times reflections about the cell centre). The quiescent box
    is invariant under them -- cubic cells, the staggered grid's faces and nodes map to
    faces and nodes, the schemes are centred, the gas is at rest -- so a particle at in-cell
    offset o moving along d has the image's disturbance: new axis a takes old axis P[a],
    offsets o'[a] = o[P[a]] (1 - o[P[a]] when reflected), the slip direction and the
    velocity targets as vectors (sign S[a]), the temperature target and the scalar
    features unchanged."""
    if copies <= 0:
        return f, y
    rng = np.random.default_rng(seed)
    fs, ys = [f], [y]
    rows = np.arange(len(f))[:, None]
    for _ in range(copies):
        P = _PERMS[rng.integers(0, 6, len(f))]
        S = 1.0 - 2.0 * ((rng.integers(0, 8, len(f))[:, None] >> np.arange(3)) & 1)
        g = f.copy()
        o = f[:, :3][rows, P]
        g[:, :3] = np.where(S < 0, 1.0 - o, o)
        g[:, 3:6] = f[:, 3:6][rows, P] * S
        z = y.copy()
        z[:, :3] = y[:, :3][rows, P] * S
        fs.append(g)
        ys.append(z)
    return np.concatenate(fs), np.concatenate(ys)


def train(f: np.ndarray, y: np.ndarray, steps: int = 20000, batch: int = 8192, lr: float = 1e-3, seed: int = 0,
          emphasis: float = 0.0, symmetries: int = 0, decay: float = 0.0):
    """Adam on the mean squared error of the targets in units of the prior. emphasis > 0 draws
    the training rows with probability proportional to prior ** emphasis (seeded), so that the
    particles with the largest disturbance per unit slip -- whose error dominates the
    self-induced slip error -- weigh more. symmetries > 0 adds that many images of every
    sample under the box's symmetries (symmetry_images). decay > 0 runs that fraction of the
    steps, at the end, at lr / 10 (Adam's moments carry over)."""
    f, y = symmetry_images(f, y, symmetries, seed + 29)
    shift, scale, lo, hi = normaliser(f)
    pr = prior(f)
    if emphasis > 0:
        w = pr ** emphasis
        pick = np.random.default_rng(seed + 17).choice(len(f), size=len(f), p=w / w.sum())
        f, y, pr = f[pick], y[pick], pr[pick]
    x = ((f - shift) * scale).astype(np.float32)
    net = mlp.Mlp(seed=seed)
    # targets in units of the prior; a few samples with a near-zero drive temperature
    # difference give meaningless ratios, which are clipped
    yt = np.clip(y / pr[:, None], -TARGET_CLIP, TARGET_CLIP)
    net.set_data(x, yt.astype(np.float32))
    late = int(round(steps * decay))
    loss = net.train(steps - late, batch=batch, lr=lr, seed=seed + 1)
    if late:
        loss = np.concatenate([loss, net.train(late, batch=batch, lr=lr * 0.1, seed=seed + 2)])
    model = dict(params=net.params, shift=shift.astype(np.float32), scale=scale.astype(np.float32),
                 lo=lo.astype(np.float32), hi=hi.astype(np.float32), prior_re=np.float32(PRIOR_RE))
    return model, loss, net


def errors(spec: Spec, rec: dict) -> dict:
    """Self-induced errors of the gas state the step used (truth: u = 0, T = 1): the gas velocity
    in units of the particle's terminal slip, the gas temperature in units of its steady excess
    temperature Q tau_T (particles with Q > 0.05); and the settling error of the final velocity."""
    c = rec["const"]
    fl = rec["flag"]
    gasv = np.stack([rec["ug"], rec["vg"], rec["wg"]], axis=1)
    s0 = np.linalg.norm(c["slip0"][fl], axis=1)
    e_slip = np.linalg.norm(gasv, axis=1) / s0
    fin = rec["final"]
    ff = fin["flag"].astype(np.int64)
    uf = np.stack([fin["u"], fin["v"], fin["w"]], axis=1)
    e_settle = np.linalg.norm(uf - c["slip0"][ff], axis=1) / np.linalg.norm(c["slip0"][ff], axis=1)
    q = c["q"][fl]
    hot = q > 0.05
    e_t = np.abs(rec["Tg"][hot] - 1.0) / (q[hot] * spec.tau_t)
    return dict(slip_rms=float(np.sqrt(np.mean(e_slip ** 2))), settle_rms=float(np.sqrt(np.mean(e_settle ** 2))),
                temp_rms=float(np.sqrt(np.mean(e_t ** 2))))


K_BINS = (0.0, 0.1, 0.3, 0.6, 0.9, float("inf"))


def per_particle_slip(rec: dict) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Per particle id of a recorded run: the RMS over its samples of the self-induced slip
    error (|gas velocity used| / terminal slip, as `errors`), and its mean K = |gas velocity
    used| / |drive slip| (the disturbance per unit slip; meaningful in a plain run, where the
    gas used is the disturbance itself)."""
    c = rec["const"]
    fl = rec["flag"]
    gasv = np.stack([rec["ug"], rec["vg"], rec["wg"]], axis=1)
    up = np.stack([rec["u"], rec["v"], rec["w"]], axis=1)
    g = np.linalg.norm(gasv, axis=1)
    s0 = np.linalg.norm(c["slip0"][fl], axis=1)
    sd = np.linalg.norm(up - gasv, axis=1)
    ids = np.unique(fl)
    e2 = np.bincount(fl, weights=(g / s0) ** 2, minlength=ids.max() + 1)
    k = np.bincount(fl, weights=np.where(sd > 0, g / np.maximum(sd, 1e-300), 0.0), minlength=ids.max() + 1)
    cnt = np.bincount(fl, minlength=ids.max() + 1)
    return ids, np.sqrt(e2[ids] / cnt[ids]), k[ids] / cnt[ids]


def slip_by_k(pairs: list[tuple[dict, dict]]) -> list[dict]:
    """Self-induced slip error of plain and corrected runs of the same particles, binned by
    the particle's K (from its plain run): RMS per bin and the reduction."""
    ep, ec, kk = [], [], []
    for plain, corr in pairs:
        ids_p, e_p, k_p = per_particle_slip(plain)
        ids_c, e_c, _ = per_particle_slip(corr)
        _, ip, ic = np.intersect1d(ids_p, ids_c, return_indices=True)
        ep.append(e_p[ip])
        ec.append(e_c[ic])
        kk.append(k_p[ip])
    ep, ec, kk = np.concatenate(ep), np.concatenate(ec), np.concatenate(kk)
    out = []
    for lo, hi in zip(K_BINS[:-1], K_BINS[1:]):
        m = (kk >= lo) & (kk < hi)
        if not m.any():
            continue
        p, c = float(np.sqrt(np.mean(ep[m] ** 2))), float(np.sqrt(np.mean(ec[m] ** 2)))
        out.append(dict(k_lo=lo, k_hi=hi, particles=int(m.sum()), plain=p, corrected=c,
                        reduction=p / max(c, 1e-300)))
    return out


def save_model(model: dict, path: str = MODEL_FILE, meta: dict | None = None):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, **{k: np.asarray(v) for k, v in model.items()}, meta=json.dumps(meta or {}))


def load_model(path: str = MODEL_FILE) -> dict:
    z = np.load(path)
    return {k: z[k] for k in ("params", "shift", "scale", "lo", "hi", "prior_re", "drive_cap") if k in z}


def pipeline(spec: Spec | None = None, seed: int = 3001, eval_seed: int = 4001, eval_runs: int | None = None,
             steps: int = 20000, batch: int = 8192, lr: float = 1e-3, eval_lattice: int = 32, rounds: int = 2,
             emphasis: float = 0.0, drive_cap: float = 0.0, symmetries: int = 0, decay: float = 0.0,
             closed_only: bool = False, log=print) -> dict:
    """Generate the training set, train, and compare plain and corrected steps on held-out boxes.

    Data: the plain two-way-coupled runs, then `rounds` times the same boxes run with the
    correction of a network trained on all data so far (the states the corrected step visits,
    with the true disturbance from the gas fields); the final network is trained on all of it
    (steps Adam steps, batch, lr).

    The held-out boxes draw particles from the same distributions at eval_lattice spacing (64 per
    128^3 box at 32 dx): the error then measures each particle's self-induced disturbance, with
    its neighbours' far fields (which decay only as 1/r in the diffusive boxes and which no
    self-correction removes) well below it. 16 dx spacing is reported too (eval_lattice=16)."""
    spec = spec or Spec()
    runs = sample(spec, seed)
    f_all, y_all = [], []
    for r, run in enumerate(runs):
        f, y, _ = raw_features(spec, run_box(spec, run))
        f_all.append(f)
        y_all.append(y)
        log(f"plain box {r}: nu {run['nu']:.3e}, {len(f)} samples")
    net_model = None
    for rnd in range(rounds):
        net_model, loss1, _ = train(np.concatenate(f_all), np.concatenate(y_all), steps=steps // 2, batch=batch, lr=lr,
                                    seed=seed + 100 * rnd, emphasis=emphasis, symmetries=symmetries, decay=decay)
        if drive_cap > 0:
            net_model["drive_cap"] = np.float32(drive_cap)
        log(f"round {rnd} network: loss {loss1[-100:].mean():.4e}")
        for r, run in enumerate(runs):
            f, y, _ = raw_features(spec, run_box(spec, run, net_model))
            f_all.append(f)
            y_all.append(y)
        log(f"round {rnd}: closed-loop samples from {len(runs)} boxes")
    if closed_only and rounds > 0:
        # the final network on the closed-loop rounds alone: in the plain runs the drag slip
        # falls as the disturbance builds up, so the disturbance per unit of the current
        # slip carries the force's history; the corrected step holds the slip steady
        f_all, y_all = f_all[len(runs):], y_all[len(runs):]
    f = np.concatenate(f_all)
    y = np.concatenate(y_all)
    model, loss, net = train(f, y, steps=steps, batch=batch, lr=lr, seed=seed + 7, emphasis=emphasis,
                             symmetries=symmetries, decay=decay)
    if drive_cap > 0:
        model["drive_cap"] = np.float32(drive_cap)
    log(f"trained: loss {loss[:10].mean():.4e} -> {loss[-100:].mean():.4e}")
    out = evaluate(model, spec, eval_seed, eval_lattice, eval_runs, log)
    out["samples"] = int(len(f))
    out["final_loss"] = float(loss[-100:].mean())
    out["model"] = model
    return out


def evaluate(model: dict, spec: Spec | None = None, seed: int = 4001, lattice: int = 32, runs: int | None = None,
             log=print, every_stage: bool = False) -> dict:
    """Plain against corrected step on held-out quiescent boxes (particles from the training
    distributions, `lattice` spacing): RMS over the boxes of each error of `errors`.
    every_stage: the network runs at every stage instead of once per step."""
    spec = spec or Spec()
    espec = dataclasses.replace(spec, lattice=lattice)
    held = sample(espec, seed)
    pick = range(espec.runs) if runs is None else [int(round(i * (espec.runs - 1) / max(runs - 1, 1)))
                                                    for i in range(runs)]
    res = {"plain": [], "corrected": []}
    per_box = []
    pairs = []
    for r in pick:
        recs = {name: run_box(espec, held[r], m, every_stage=every_stage)
                for name, m in (("plain", None), ("corrected", model))}
        pairs.append((recs["plain"], recs["corrected"]))
        e = {name: errors(espec, rec) for name, rec in recs.items()}
        for name in res:
            res[name].append(e[name])
        per_box.append(dict(box=r, nu=held[r]["nu"], **{f"{n}_{k}": v for n in e for k, v in e[n].items()}))
        log(f"held-out box {r} (nu {held[r]['nu']:.2e}): plain {e['plain']} corrected {e['corrected']}")
    out = {}
    for name in res:
        out[name] = {k: float(np.sqrt(np.mean([e[k] ** 2 for e in res[name]]))) for k in res[name][0]}
    out["slip_reduction"] = out["plain"]["slip_rms"] / max(out["corrected"]["slip_rms"], 1e-300)
    out["settle_reduction"] = out["plain"]["settle_rms"] / max(out["corrected"]["settle_rms"], 1e-300)
    out["temp_reduction"] = out["plain"]["temp_rms"] / max(out["corrected"]["temp_rms"], 1e-300)
    out["boxes"] = per_box
    out["slip_by_k"] = slip_by_k(pairs)
    return out


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="train the learned correction on quiescent-gas runs")
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--rounds", type=int, default=2, help="closed-loop data rounds before the final training")
    ap.add_argument("--emphasis", type=float, default=0.0, help="draw training rows with probability prior**emphasis")
    ap.add_argument("--drive-cap", type=float, default=0.0, help="drive slip cap in units of the plain slip (0: 10)")
    ap.add_argument("--symmetries", type=int, default=0, help="images of each sample under the box's symmetries")
    ap.add_argument("--decay", type=float, default=0.0, help="fraction of the steps run at lr/10 at the end")
    ap.add_argument("--closed-only", action="store_true", help="final network on the closed-loop rounds' data only")
    ap.add_argument("--out", default=MODEL_FILE)
    a = ap.parse_args()
    r = pipeline(steps=a.steps, rounds=a.rounds, emphasis=a.emphasis, drive_cap=a.drive_cap, symmetries=a.symmetries,
                 decay=a.decay, closed_only=a.closed_only)
    meta = {k: r[k] for k in ("plain", "corrected", "slip_reduction", "settle_reduction", "temp_reduction", "samples",
                              "final_loss", "boxes", "slip_by_k")}
    meta["settings"] = {"steps": a.steps, "rounds": a.rounds, "emphasis": a.emphasis, "drive_cap": a.drive_cap,
                        "symmetries": a.symmetries, "decay": a.decay, "closed_only": a.closed_only}
    save_model(r["model"], a.out, meta)
    print(json.dumps(meta))

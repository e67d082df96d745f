"""Physical configuration of the particle step and the named workloads.

The reference reads a positional parameter file (params.cpp:22-48) and derives
Tp, mp, R, P0, N0 from it (params.cpp:51-56). The step itself only needs the
derived scalars below; `derive()` computes them with the reference's own
expression order so that host-side values are bit-identical to what the
reference's params class would hold.
"""
from __future__ import annotations

import dataclasses
import math

PI = 3.141592653589793  # params.h:5
RK4_PRE = (0.5, 0.5, 1.0, 1.0 / 6.0)  # grid.cpp:16-19
RK4_POST = (1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0)  # grid.cpp:20-23


@dataclasses.dataclass
class BoxParams:
    """Raw parameter-file values for a periodic box (params.h names)."""
    n: int
    l: float
    dt: float
    rho0: float
    t0: float
    mu0: float
    k: float
    cp: float
    cv: float
    np0: float
    dp: float
    rhop: float
    cvp: float
    epsilonp: float
    nu: float
    i0: float
    gx: float = 0.0
    gy: float = 0.0
    gz: float = 0.0
    twc: int = 1
    particle_gravity: int = 0
    # gas-step settings (params.in lines Cooling, iterations/convergence, A1 A2, U0)
    cooling: int = 0
    iterations: int = 30
    epsilon: float = 1e-7
    a_force: float = 0.0
    u0: float = 0.0

    def derived(self) -> dict:
        """params.cpp:51-56 in the reference's operand order."""
        r = self.cp - self.cv
        return {
            "R": r,
            "P0": self.rho0 * self.t0 * r,
            "Tp": self.rhop * self.dp * self.dp / (18 * self.mu0),
            "mp": self.rhop * PI * self.dp * self.dp * self.dp / 6.0,
            "N0": int(self.np0 * (self.l * self.l * self.l)),
        }

    def step_config(self) -> dict:
        """The scalars the particle step consumes (the C-ABI's pstep_config fields)."""
        d = self.derived()
        return dict(n=self.n, l=self.l, dt=self.dt, tp=d["Tp"], mp=d["mp"], dp=self.dp, nu=self.nu, k=self.k,
                    epsilonp=self.epsilonp, i0=self.i0, cvp=self.cvp, gx=self.gx, gy=self.gy, gz=self.gz,
                    particle_gravity=self.particle_gravity, twc=self.twc)

    def gas_config(self) -> dict:
        """The scalars the box gas step consumes (grid.cpp; params.cpp:22-56)."""
        d = self.derived()
        return dict(n=self.n, l=self.l, dt=self.dt, mu0=self.mu0, k=self.k, cp=self.cp, cv=self.cv, rho0=self.rho0,
                    u0=self.u0, a_force=self.a_force, gx=self.gx, gy=self.gy, gz=self.gz, mp=d["mp"],
                    epsilon=self.epsilon, iterations=self.iterations, cooling=self.cooling, twc=self.twc,
                    p0=d["P0"])

    def params_file(self) -> str:
        """A parameter file in the reference's positional format (params.cpp:22-48)."""
        r = repr
        lines = [
            "1", f"{self.n} {self.n} {self.n}", f"{r(self.l)} {r(self.l)} {r(self.l)}", "1", "0",
            f"1 {r(self.dt)} 1e30", "0 0", "1000000 1000000", "./ ./", "2", "0 0", str(self.cooling),
            f"{self.iterations} {self.iterations} {r(self.epsilon)}",
            f"{self.twc} {self.particle_gravity}", f"{r(self.a_force)} {r(self.a_force)}", r(self.rho0),
            r(self.u0), r(self.t0),
            f"{r(self.mu0)} {r(self.k)}",
            f"{r(self.gx)} {r(self.gy)} {r(self.gz)} {r(self.gx)} {r(self.gy)} {r(self.gz)}",
            f"{r(self.cp)} {r(self.cv)}", r(self.np0), f"{r(self.dp)} {r(self.rhop)}", r(self.cvp),
            r(self.epsilonp), r(self.nu), f"{r(self.i0)} {r(self.i0)}",
        ]
        return "\n".join(lines) + "\n"


def box_params(n: int, n_particles: int, *, l: float = 2 * PI, dp_over_dx: float = 0.1,
               mass_loading: float = 0.2, tau_p: float = 0.1, tau_t: float = 0.15, q: float = 1.0,
               nu: float = 2.0, k: float = 1.0, epsilonp: float = 1.0, dt: float = 1e-3,
               twc: int = 1) -> BoxParams:
    """Nondimensional box: rho0 = T0 = 1 so P0/R = 1 and T = 1/rho; particle
    properties chosen so that tau_p, tau_T, the heating rate Q = alpha*iS and
    the mass loading N0*mp/(Vol*rho0) take the requested values."""
    dx = l / n
    dp = dp_over_dx * dx
    vol = l * l * l
    mp = mass_loading * vol * 1.0 / n_particles
    rhop = 6 * mp / (PI * dp ** 3)
    mu0 = rhop * dp * dp / (18 * tau_p)
    cvp = tau_t * nu * PI * dp * k / mp
    i0 = q * mp * cvp / (0.25 * epsilonp * PI * dp * dp)
    np0 = (n_particles + 0.5) / vol
    return BoxParams(n=n, l=l, dt=dt, rho0=1.0, t0=1.0, mu0=mu0, k=k, cp=3.5, cv=2.5, np0=np0, dp=dp,
                     rhop=rhop, cvp=cvp, epsilonp=epsilonp, nu=nu, i0=i0, twc=twc)


@dataclasses.dataclass
class Workload:
    name: str
    n: int
    n_particles: int
    clustered: bool
    steps: int
    seed: int
    dp_over_dx: float = 0.1
    mass_loading: float = 0.2
    nblobs: int = 64  # Gaussian blobs holding the clustered half of the particles (sigma 4 cells)
    tau_p_range: tuple | None = None  # per-particle tau_p, log-uniform in [lo, hi] (None: the scalar)

    def tau_p(self):
        """The per-particle momentum relaxation times of the workload (None: scalar tau_p)."""
        if self.tau_p_range is None:
            return None
        from . import gen
        return gen.loguniform(self.seed, 31, self.n_particles, *self.tau_p_range)


# Seeded synthetic stand-ins for the reference's run shapes.
WORKLOADS = {
    "box64_uniform": Workload("box64_uniform", 64, 1 << 15, False, 1, 1001),
    "box256_clustered": Workload("box256_clustered", 256, 1 << 24, True, 10, 1002),
    "box512_clustered": Workload("box512_clustered", 512, 1 << 27, True, 1, 1003),
    # the mixed-precision configuration: box512_clustered's construction with tau_p
    # log-uniform in [0.01, 1] per particle, for the FP32 form's error against FP64
    "box512_mixed": Workload("box512_mixed", 512, 1 << 27, True, 1, 1006, tau_p_range=(0.01, 1.0)),
    # the corrected-step workload: larger, heavier particles (d_p/dx 0.5, mass loading 1.0)
    "box512_corrected": Workload("box512_corrected", 512, 1 << 27, True, 100, 1004, 0.5, 1.0),
    # box512_corrected at 1/8 of the cells and particles with 8 blobs instead of 64: each
    # blob holds 2^20 particles as there, so the cell occupancy (up to ~1000 particles
    # in a blob-centre cell, 44% of the particles in cells holding 64 or more) is the
    # same; the profiling case for the deposit
    "box256_dense": Workload("box256_dense", 256, 1 << 24, True, 1, 1005, 0.5, 1.0, 8),
}


def mass_loading_check(bp: BoxParams, n_particles: int) -> float:
    """params.h:98 St(): N0*mp/(Vol*Rho0)."""
    d = bp.derived()
    return n_particles * d["mp"] / (bp.l ** 3 * bp.rho0)


def heating_rate(bp: BoxParams) -> float:
    """alpha * iS of particle.cpp:484-486."""
    d = bp.derived()
    alpha = 0.25 * bp.epsilonp * PI * bp.dp * bp.dp * bp.i0
    return alpha * (1.0 / (d["mp"] * bp.cvp))


def tau_t(bp: BoxParams) -> float:
    d = bp.derived()
    return d["mp"] * bp.cvp / (bp.nu * PI * bp.dp * bp.k)


__all__ = ["PI", "RK4_PRE", "RK4_POST", "BoxParams", "box_params", "Workload", "WORKLOADS", "math"]

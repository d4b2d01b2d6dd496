"""Seeded synthetic workloads of the batched and served configurations.

The reference has no test case with a tilted planar or a random-state circular Sod interface; the
initial states below are written in the reference's array layout (init_test's cell-centre rule,
src/kernels/init_test.cpp:65-93) and fed identically to the GPU and to the oracle.

Mixed batch (configuration 3): `mixed_domains(256, seed)` draws, per domain, sides nx, ny from
{64, 128, ..., 1024} independently; a planar or circular interface with position
pos ~ U(0.3, 0.7); left/high state rho ~ U(0.5, 2), p ~ U(0.5, 2); right/low state rho ~ U(0.05, 0.3),
p ~ U(0.05, 0.3); u = v = 0; E = p / ((gamma - 1) rho); angle ~ U(0, pi).
  planar:   high state where (x - 0.5, y - 0.5) . (cos a, sin a) <= pos - 0.5
  circular: high state where |(x, y) - (0.5, 0.5)| <= pos / 2
Every domain: [0, 1]^2, reflective walls (Sod_circ's boundary factors), GAD-minmod, euler_2nd,
5 ghosts, CFL 0.6, run to t = 0.15.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import Case, Params, SodInterface, make_params

GAMMA = 1.4
SIDES = (64, 128, 256, 512, 1024)


@dataclass
class DomainSpec:
    nx: int
    ny: int
    kind: str          # "planar" or "circular"
    pos: float
    angle: float
    rho_l: float
    rho_r: float
    p_l: float
    p_r: float
    t_end: float = 0.15
    precision: int = 64
    splitting: str = "Sequential"

    def case(self) -> Case:
        return Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", limiter="Minmod", nghost=5,
                    nx=self.nx, ny=self.ny, cfl=0.6, max_time=self.t_end, max_cycles=1_000_000,
                    splitting=self.splitting)

    def params(self) -> Params:
        return make_params(self.case())

    def initial_state(self) -> dict[str, np.ndarray]:
        """rho, umat, vmat, Emat over all nb_cells cells (ghosts included)."""
        p = self.params()
        g, R, Cl = p.nb_ghosts, p.row_length, p.col_length
        ix = np.arange(R) - g
        iy = np.arange(Cl) - g
        # cell centres as init_test computes them: x = ix / nx * sx + ox, centre = x + sx / (2 nx)
        xm = ix / self.nx * 1.0 + 0.0 + 1.0 / (2 * self.nx)
        ym = iy / self.ny * 1.0 + 0.0 + 1.0 / (2 * self.ny)
        X, Y = np.meshgrid(xm, ym)
        if self.kind == "planar":
            high = (X - 0.5) * np.cos(self.angle) + (Y - 0.5) * np.sin(self.angle) <= self.pos - 0.5
        else:
            high = (X - 0.5) ** 2 + (Y - 0.5) ** 2 <= (self.pos / 2) ** 2
        rho = np.where(high, self.rho_l, self.rho_r)
        pr = np.where(high, self.p_l, self.p_r)
        E = pr / ((GAMMA - 1) * rho)
        z = np.zeros_like(rho)
        return {"rho": rho.ravel(), "umat": z.ravel(), "vmat": z.ravel().copy(), "Emat": E.ravel()}

    def sod_interface(self) -> SodInterface:
        """The same initial state made on the device (armon_sod_interface): every operand and operation
        of initial_state's tests, in the same order."""
        s = SodInterface()
        s.cx = s.cy = 0.5
        if self.kind == "planar":
            s.shape = 0
            s.nx, s.ny = float(np.cos(self.angle)), float(np.sin(self.angle))
            s.offset = self.pos - 0.5
        else:
            s.shape = 1
            s.r2 = (self.pos / 2) ** 2
        s.rho_high, s.p_high, s.rho_low, s.p_low = self.rho_l, self.p_l, self.rho_r, self.p_r
        return s

    @property
    def cells(self) -> int:
        return self.nx * self.ny


def mixed_domains(n: int = 256, seed: int = 2024, sides=SIDES) -> list[DomainSpec]:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        out.append(DomainSpec(nx=int(rng.choice(sides)), ny=int(rng.choice(sides)),
                              kind="planar" if rng.random() < 0.5 else "circular",
                              pos=float(rng.uniform(0.3, 0.7)), angle=float(rng.uniform(0, np.pi)),
                              rho_l=float(rng.uniform(0.5, 2.0)), rho_r=float(rng.uniform(0.05, 0.3)),
                              p_l=float(rng.uniform(0.5, 2.0)), p_r=float(rng.uniform(0.05, 0.3))))
    return out


@dataclass
class Request:
    arrival: float        # seconds after the start of the trace
    spec: DomainSpec


def serving_trace(n: int = 10_000, rate: float = 50.0, seed: int = 7, mu: float = 6.0, sigma: float = 0.6,
                  side_range=(128, 2048)) -> list[Request]:
    """Poisson arrivals at `rate` per second; side ~ lognormal(mu, sigma) clipped to side_range and
    rounded to a multiple of 16; FP64 or FP32 with probability 1/2; final time ~ U(0.05, 0.2); the
    interface drawn as in mixed_domains (configuration 4)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(n):
        t += float(rng.exponential(1.0 / rate))
        side = int(np.clip(rng.lognormal(mu, sigma), *side_range)) // 16 * 16
        side = max(side, side_range[0])
        spec = DomainSpec(nx=side, ny=side, kind="planar" if rng.random() < 0.5 else "circular",
                          pos=float(rng.uniform(0.3, 0.7)), angle=float(rng.uniform(0, np.pi)),
                          rho_l=float(rng.uniform(0.5, 2.0)), rho_r=float(rng.uniform(0.05, 0.3)),
                          p_l=float(rng.uniform(0.5, 2.0)), p_r=float(rng.uniform(0.05, 0.3)),
                          t_end=float(rng.uniform(0.05, 0.2)), precision=64 if rng.random() < 0.5 else 32)
        out.append(Request(arrival=t, spec=spec))
    return out

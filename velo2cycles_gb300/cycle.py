"""Seismic-cycle step sequence on the GPU pipeline (the config-1 geometry run
for many steps with the time step switching between an interseismic and a
coseismic regime).

The reference gets each step's velocities from its Stokes solve (Pardiso,
outside the marker path).  Here a prescribed-velocity stand-in takes its
place: regime 0 uses the loading field of the synthetic case, regime 1 adds
a slip pulse across the frictional band (a divergence-free shear from the
stream function psi = V/2 w log cosh((y - y_f)/w)).  Events are nucleated
after a fixed number of interseismic steps and the pulse stops once its slip
budget is spent.  The pulse steps are coseismic; otherwise the time step
follows the pipeline's own maximum slip rate from calc_timestep
(calc_RSF.c:352-572): coseismic dt while the rate exceeds `v_switch` (for at
most `relax_max` steps after an event), interseismic dt below it.  Each (regime, dt) pair runs as a captured CUDA
graph (v2c_cycle_step).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import abi


@dataclass
class Schedule:
    dt_inter: float = 1e9        # s
    dt_co: float = 1e-3          # s
    v_switch: float = 1e-3       # m/s, slip rate that selects the coseismic dt
    n_inter: int = 150           # interseismic steps before an event
    v_pulse: float = 1.0         # m/s across the band during an event
    width: float = 1000.0        # m, half-width of the pulse shear zone
    slip_budget: float = 0.1     # m of pulse slip per event
    relax_max: int = 50          # coseismic-dt steps after a pulse at most


def pulse_fields(case, s: Schedule):
    """(vx, vy) of the loading field and of loading + slip pulse on the
    staggered velocity nodes of `case` (vx nodes at (gx[i], mid y), vy nodes
    at (mid x, gy[j]))."""
    gx, gy = case.gx, case.gy
    xn, yn = gx.size, gy.size
    I, J = np.meshgrid(np.arange(xn), np.arange(yn), indexing="ij")
    I, J = I.ravel(), J.ravel()
    Jp = np.minimum(J + 1, yn - 1)
    Ip = np.minimum(I + 1, xn - 1)
    xvx, yvx = gx[I], 0.5 * (gy[J] + gy[Jp])
    xvy = 0.5 * (gx[I] + gx[Ip])
    p = case.params
    yf, sl = p["fault_y"], p["fault_slope"]
    vx0, vy0 = case.nodes[abi.NF_VX].copy(), case.nodes[abi.NF_VY].copy()
    # psi = V/2 w log cosh(d/w), d = y - yf - sl x: vx = dpsi/dy, vy = -dpsi/dx
    vx1 = vx0 + 0.5 * s.v_pulse * np.tanh((yvx - yf - sl * xvx) / s.width)
    vy1 = vy0 + 0.5 * s.v_pulse * sl * np.tanh((gy[J] - yf - sl * xvy) / s.width)
    return (vx0, vy0), (vx1, vy1)


@dataclass
class Record:
    regime: list = field(default_factory=list)
    dt: list = field(default_factory=list)
    maxvel: list = field(default_factory=list)
    seconds: float = 0.0


class Driver:
    """Regime and time-step decisions over a stepper with
    cycle_step(regime, dt) and calc_timestep(oldornew) -> info dict."""

    def __init__(self, s: Schedule):
        self.s = s
        self.regime = 0
        self.dt = s.dt_inter
        self.n_in_regime = 0
        self.n_relax = 0
        self.slip = 0.0

    def next(self, maxvel: float):
        """Advance the decisions after a step whose maximum slip rate was
        maxvel; returns (regime, dt) of the next step.  While the pulse runs
        the step is coseismic; afterwards dt follows the slip rate for at most
        `relax_max` steps (the stand-in has no healing: with a coseismic dt
        simulated time hardly advances), and only interseismic steps count
        towards the next event."""
        s = self.s
        if self.regime == 1:
            self.slip += s.v_pulse * self.dt
            if self.slip < s.slip_budget:
                return self.regime, self.dt
            self.regime, self.n_in_regime, self.n_relax = 0, 0, 0
        elif self.dt == s.dt_inter:
            self.n_in_regime += 1
            if self.n_in_regime >= s.n_inter:
                self.regime, self.slip, self.dt = 1, 0.0, s.dt_co
                return self.regime, self.dt
        co = maxvel > s.v_switch and self.n_relax < s.relax_max
        self.n_relax = self.n_relax + 1 if co else s.relax_max
        self.dt = s.dt_co if co else s.dt_inter
        return self.regime, self.dt


def run(stepper, s: Schedule, steps: int, forced=None) -> Record:
    """Run `steps` cycle steps.  forced: a list of (regime, dt) to replay
    instead of deciding (the same sequence on two arithmetic forms)."""
    rec = Record()
    drv = Driver(s)
    regime, dt = 0, s.dt_inter
    t0 = time.perf_counter()
    for k in range(steps):
        if forced is not None:
            regime, dt = forced[k]
        stepper.cycle_step(regime, dt)
        info = stepper.calc_timestep(1)
        rec.regime.append(regime)
        rec.dt.append(dt)
        rec.maxvel.append(float(info["maxvel"]))
        if forced is None:
            regime, dt = drv.next(float(info["maxvel"]))
    rec.seconds = time.perf_counter() - t0
    return rec

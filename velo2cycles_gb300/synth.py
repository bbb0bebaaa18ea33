"""Seeded synthetic marker-in-cell states in the reference's array layout.

The reference ships no benchmark inputs and its initial-condition generator
(src/in2evps.c) needs .t3c model files; these generators build states of the
same form directly, with the shapes of the benchmark configurations:

* ``c1``  301 x 101 uniform grid (600 x 200 km, 2 km), 4 x 4 markers per cell
  jittered inside sub-cells (src/in2evps.c:987-988), layered crust/mantle with
  a slab dipping 15 degrees, half-space-cooling temperature
  (src/in2evps.c:1245-1246), stream-function velocity (~5 cm/yr) plus a 2 km
  Gaussian shear band along the megathrust; dt = 1e8 s.
* ``c2``  1001 x 401 non-uniform grid refined to 100 m in a 20 km zone
  (ramp as in src/in2evps.c:847-862), 16 markers per cell, marker stress
  N(0, 5 MPa), strain rate log-uniform 1e-18..1e-10 1/s.
* ``c4``  4001 x 1001 uniform grid, 20 markers per cell (5 x 4).
* ``small`` / ``tiny``  reduced grids with the c1 physics, for tests.

The rock table is synthetic (the reference ships two Newtonian rocks only):
type 2 sediment (Newtonian), 3 upper crust, 4 lower crust and 5 mantle
(power-law creep, exercising density_ductilevisc_calc.c:65-200), 6 slab
(Newtonian).  Type 0 is unused and all-zero.  Node fields that the Stokes
solver would produce are smooth analytic fields with seeded perturbations.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi

# ----------------------------------------------------------------- params

def default_params(**kw) -> dict:
    """Flags and scalars of the shipped configuration (src/mode_RSF.t3c,
    src/input_RSF.c:13-63)."""
    p = dict(
        xnumx=0, ynumy=0, xsize=0.0, ysize=0.0, xstpx=0.0, ystpy=0.0,
        timesum=1.0e12, timestep=1.0e8,
        interpolationmod=2, antidiffinter=1, markmod=2, stoksmod=1, outgrid=2,
        densimod=0, RSFmode=1, power_law_RSF=0, rkmod=0, stickymod=1,
        inertyn=0, pmode=0, tempmod=1, compressiblemode=0, reloadfromDP=0,
        nubeg=1e1, nuend=1.667e27, nstress=10.0e6, Dphis=0.0,
        zdeep=3000000.0, tdeep=1873.0, eps2=273.0,
        a_vw=0.009, b_vw=0.017, L_vw=0.0100, V0_vw=4.0e-09,
        a_vs=0.020, b_vs=0.001, L_vs=0.0100, V0_vs=4.0e-09,
        a_hr=0.009, b_hr=0.017, L_hr=0.0100, V0_hr=4.0e-09,
        start_updip=8.0e3, end_updip=12.0e3, start_downdip=38.0e3,
        end_downdip=42.0e3, half_range=2.0e3,
        fault_y=10.0e3, fault_hw=100.0, fault_slope=0.0,
        faultwidth=400.0, newton_rtol=1e-10, newton_maxit=60,
        newton_guess=0, newton_precision=0,
    )
    p.update(kw)
    return p


def rock_table() -> np.ndarray:
    """Synthetic rock table rt[V2C_RT_N][200]."""
    rt = np.zeros((abi.RT_N, abi.MAXTMR), dtype=np.float64)

    def rock(t, gg, nu, dh=0.0, dv=0.0, ss=0.0, mm=1.0, ro=3000.0, bb=3e-5,
             aa=1e-3, cp=1000.0, kt=2.0, kf=0.0, kp=0.0, ht=0.0, n0=1e17, n1=1e26):
        rt[abi.RT_GG, t], rt[abi.RT_NU, t], rt[abi.RT_DH, t] = gg, nu, dh
        rt[abi.RT_DV, t], rt[abi.RT_SS, t], rt[abi.RT_MM, t] = dv, ss, mm
        rt[abi.RT_RO, t], rt[abi.RT_BB, t], rt[abi.RT_AA, t] = ro, bb, aa
        rt[abi.RT_CP, t], rt[abi.RT_KT, t], rt[abi.RT_HT, t] = cp, kt, ht
        rt[abi.RT_KF, t], rt[abi.RT_KP, t] = kf, kp
        rt[abi.RT_N0, t], rt[abi.RT_N1, t] = n0, n1

    # sediment, Newtonian
    rock(2, 3.0e10, 1.0e21, ro=2400.0, kt=1.5, kf=300.0, kp=4e-5, ht=1.5e-6)
    # upper crust, wet-quartzite-like dislocation creep
    rock(3, 3.0e10, 1.7e21, dh=1.50e5, dv=0.0, ss=1.0e6, mm=3.0, ro=2700.0,
         kt=0.64, kf=807.0, kp=4e-5, ht=1.0e-6)
    # lower crust
    rock(4, 3.0e10, 2.35e19, dh=2.40e5, dv=1.2, ss=1.0e6, mm=3.2, ro=2900.0,
         kt=1.18, kf=474.0, kp=4e-5, ht=2.5e-7)
    # mantle, olivine-like
    rock(5, 6.7e10, 1.08e18, dh=5.30e5, dv=1.5, ss=3.0e6, mm=3.5, ro=3300.0,
         kt=0.73, kf=1293.0, kp=4e-5, ht=2.2e-8)
    # slab (oceanic crust), Newtonian
    rock(6, 3.5e10, 1.0e23, ro=3000.0, kt=1.18, kf=474.0, kp=4e-5, ht=2.5e-7)
    return rt


# ------------------------------------------------------------------- case

@dataclass
class Case:
    name: str
    params: dict
    gx: np.ndarray
    gy: np.ndarray
    rt: np.ndarray
    nodes: dict            # field id -> float64[nodenum]
    marks: dict            # field id -> float64[n]
    markt: np.ndarray      # int8[n]
    bondm: np.ndarray      # int64[nodenum*4]
    bondn: np.ndarray      # int64[bondnum*3]
    bondv: np.ndarray      # float64[bondnum*4]
    extra: dict = field(default_factory=dict)

    @property
    def nodenum(self) -> int:
        return int(self.params["xnumx"] * self.params["ynumy"])

    @property
    def n(self) -> int:
        return int(self.markt.shape[0])

    @property
    def bondnum(self) -> int:
        return int(self.bondv.shape[0] // 4)

    def copy(self) -> "Case":
        return Case(self.name, dict(self.params), self.gx.copy(), self.gy.copy(),
                    self.rt.copy(), {k: v.copy() for k, v in self.nodes.items()},
                    {k: v.copy() for k, v in self.marks.items()}, self.markt.copy(),
                    self.bondm.copy(), self.bondn.copy(), self.bondv.copy(),
                    dict(self.extra))


def _ramp_grid(n: int, size: float, fine: float, z0: float, z1: float) -> np.ndarray:
    """Grid lines with spacing `fine` inside [z0, z1] and a geometric ramp to
    a uniform coarse spacing outside (the refinement of src/in2evps.c:847-862),
    exactly n lines from 0 to size."""
    nf = int(round((z1 - z0) / fine))
    rest = n - 1 - nf
    left_len, right_len = z0, size - z1
    nl = max(1, int(round(rest * left_len / (left_len + right_len))))
    nr = rest - nl

    def side(m, length):
        # geometric growth from `fine` so the m steps sum to `length`
        lo, hi = 1.0, 2.0
        for _ in range(200):
            q = 0.5 * (lo + hi)
            s = fine * (q ** np.arange(1, m + 1)).sum()
            if s > length:
                hi = q
            else:
                lo = q
        st = fine * (lo ** np.arange(1, m + 1))
        return st * (length / st.sum())

    steps = np.concatenate([side(nl, left_len)[::-1], np.full(nf, fine), side(nr, right_len)])
    g = np.concatenate([[0.0], np.cumsum(steps)])
    g[-1] = size
    return g


_CONFIGS = {
    # name: xnumx, ynumy, xsize, ysize, mx, my, refine
    "tiny": (26, 14, 50e3, 26e3, 4, 4, None),
    "small": (51, 21, 100e3, 40e3, 4, 4, None),
    "c1": (301, 101, 600e3, 200e3, 4, 4, None),
    "c2": (1001, 401, 600e3, 200e3, 4, 4, (100.0, 20e3)),
    "c4": (4001, 1001, 2000e3, 500e3, 5, 4, None),
}


def grid_for(name: str):
    xn, yn, xs, ys, mx, my, refine = _CONFIGS[name]
    if refine is None:
        gx = np.linspace(0.0, xs, xn)
        gy = np.linspace(0.0, ys, yn)
    else:
        fine, width = refine
        # refined zone around the megathrust at 200-220 km along x and
        # 5-25 km in depth
        gx = _ramp_grid(xn, xs, fine, 200e3, 200e3 + width)
        gy = _ramp_grid(yn, ys, fine, 5e3, 5e3 + width)
    return gx, gy, mx, my


# -------------------------------------------------------- physical fields

SLAB_X0 = 0.33  # trench position as a fraction of xsize
DIP = math.radians(15.0)
V_PLATE = 5.0e-2 / (365.25 * 86400.0)  # 5 cm/yr


def _temperature(y, ysize):
    # half-space cooling, 60 Myr, 273 K surface, 1623 K mantle
    kappa, age = 1e-6, 60e6 * 3.15576e7
    from scipy.special import erf
    return 273.0 + (1623.0 - 273.0) * erf(y / (2.0 * math.sqrt(kappa * age)))


def _stream(x, y, xs, ys):
    """velocity, strain rate and spin of psi = A sin(pi x/Lx) sin(pi y/Ly)
    plus a Gaussian shear band along the slab top."""
    A = V_PLATE * ys / math.pi
    kx, ky = math.pi / xs, math.pi / ys
    sx, cx = np.sin(kx * x), np.cos(kx * x)
    sy, cy = np.sin(ky * y), np.cos(ky * y)
    vx = A * ky * sx * cy
    vy = -A * kx * cx * sy
    dvxdx = A * ky * kx * cx * cy
    dvxdy = -A * ky * ky * sx * sy
    dvydx = A * kx * kx * sx * sy
    # shear band: tangential velocity along the dipping line y = tan(dip)(x-x0)
    x0 = SLAB_X0 * xs
    t = np.array([math.cos(DIP), math.sin(DIP)])
    d = (y - math.tan(DIP) * (x - x0)) * math.cos(DIP)  # signed distance
    w = 1.0e3
    g = V_PLATE * np.exp(-0.5 * (d / w) ** 2) * (x > x0)
    dg_dd = -g * d / (w * w)
    # d(d)/dx = -sin(dip), d(d)/dy = cos(dip)
    vx = vx + g * t[0]
    vy = vy + g * t[1]
    dvxdx = dvxdx + t[0] * dg_dd * (-math.sin(DIP))
    dvxdy = dvxdy + t[0] * dg_dd * math.cos(DIP)
    dvydx = dvydx + t[1] * dg_dd * (-math.sin(DIP))
    exx = dvxdx
    exy = 0.5 * (dvxdy + dvydx)
    esp = 0.5 * (dvydx - dvxdy)
    return vx, vy, exx, exy, esp


def _rock_type(x, y, xs):
    t = np.full(x.shape, 5, dtype=np.int8)
    t[y < 35e3] = 4
    t[y < 15e3] = 3
    t[y < 2e3] = 2
    x0 = SLAB_X0 * xs
    top = math.tan(DIP) * (x - x0)
    inslab = (x > x0) & (y > top) & (y < top + 8e3 / math.cos(DIP))
    t[inslab] = 6
    return t


def _bonds(xn: int, yn: int, pinit: float = 10.0e6):
    """Boundary equations in the reference layout (bondm/bondn/bondv,
    src/headevps.c:205-209): plate-speed shear on the top and bottom vx rows,
    free-slip copies on the side columns, a pressure anchor at node (1,1) and
    fixed/insulating temperature sides."""
    nn = xn * yn
    bondm = np.zeros(nn * 4, dtype=np.int64)
    rows_n, rows_v = [[0, 0, 0]], [[0.0, 0.0, 0.0, 0.0]]

    def add(param, const, refs=()):
        b = len(rows_v)
        bn, bv = [0, 0, 0], [const, 0.0, 0.0, 0.0]
        for k, (rparam, coef) in enumerate(refs):
            bn[k] = rparam + 1
            bv[k + 1] = coef
        rows_n.append(bn)
        rows_v.append(bv)
        bondm[param] = b

    def m3(i, j):
        return i * yn + j

    add(m3(1, 1) * 3 + 0, pinit)
    for i in range(xn):
        add(m3(i, 0) * 3 + 1, +2.0e-9)
        add(m3(i, yn - 2) * 3 + 1, -2.0e-9)
    for j in range(yn - 1):
        add(m3(0, j) * 3 + 1, 0.0, [(m3(1, j) * 3 + 1, 1.0)])
        add(m3(xn - 1, j) * 3 + 1, 0.0, [(m3(xn - 2, j) * 3 + 1, 1.0)])
    for i in range(xn - 1):
        add(m3(i, 0) * 3 + 2, 0.0)
        add(m3(i, yn - 1) * 3 + 2, 0.0)
    for j in range(1, yn - 1):
        add(m3(0, j) * 3 + 2, 0.0, [(m3(1, j) * 3 + 2, 1.0)])
        add(m3(xn - 2, j) * 3 + 2, 0.0, [(m3(xn - 3, j) * 3 + 2, 1.0)])
    for i in range(xn):
        add(3 * nn + m3(i, 0), 273.0)
        add(3 * nn + m3(i, yn - 1), 1623.0)
    for j in range(1, yn - 1):
        add(3 * nn + m3(0, j), 0.0, [(3 * nn + m3(1, j), 1.0)])
        add(3 * nn + m3(xn - 1, j), 0.0, [(3 * nn + m3(xn - 2, j), 1.0)])
    return bondm, np.array(rows_n, dtype=np.int64).ravel(), np.array(rows_v).ravel()


def make_case(name: str = "small", seed: int = 0, n_markers: int | None = None,
              random_fields: bool | None = None, window: tuple | None = None,
              **param_overrides) -> Case:
    """Build a seeded synthetic state.  `random_fields` switches the marker
    stress/strain rate to the c2 distributions (default: only for c2).
    `window` = (i0, j0, nx, ny) cuts nx x ny grid lines starting at line
    (i0, j0) out of the configuration: same spacing, materials and fields,
    coordinates shifted so the window starts at 0 (a bounded sample of a
    large configuration)."""
    rng = np.random.default_rng(seed)
    gx, gy, mx, my = grid_for(name)
    XS, YS = float(gx[-1]), float(gy[-1])  # full model, for the physics
    ox = oy = 0.0
    if window is not None:
        i0, j0, nxw, nyw = window
        ox, oy = float(gx[i0]), float(gy[j0])
        gx = gx[i0:i0 + nxw] - ox
        gy = gy[j0:j0 + nyw] - oy
    xn, yn = gx.size, gy.size
    xs, ys = float(gx[-1]), float(gy[-1])
    nn = xn * yn
    if random_fields is None:
        random_fields = name == "c2"
    p = default_params(xnumx=xn, ynumy=yn, xsize=xs, ysize=ys,
                       xstpx=xs / (xn - 1), ystpy=ys / (yn - 1))
    p.update(param_overrides)
    rt = rock_table()

    # markers: mx x my per cell, jittered inside sub-cells
    ncx, ncy = xn - 1, yn - 1
    per = mx * my
    ncell = ncx * ncy
    n = ncell * per if n_markers is None else int(n_markers)
    ids = np.arange(n, dtype=np.int64)
    cell = (ids // per) % ncell
    sub = ids % per
    ci, cj = cell // ncy, cell % ncy
    si, sj = sub // my, sub % my
    fx = (si + rng.random(n)) / mx
    fy = (sj + rng.random(n)) / my
    x = gx[ci] + fx * (gx[ci + 1] - gx[ci])
    y = gy[cj] + fy * (gy[cj + 1] - gy[cj])
    t = _rock_type(x + ox, y + oy, XS)

    marks = {}
    marks[abi.MF_X], marks[abi.MF_Y] = x, y
    marks[abi.MF_K] = _temperature(y + oy, YS) + rng.normal(0, 5.0, n)
    mvx, mvy, mexx, mexy, _ = _stream(x + ox, y + oy, XS, YS)
    if random_fields:
        marks[abi.MF_XX] = rng.normal(0.0, 5e6, n)
        marks[abi.MF_XY] = rng.normal(0.0, 5e6, n)
        mag = 10.0 ** rng.uniform(-18, -10, n)
        ang = rng.uniform(0, 2 * math.pi, n)
        marks[abi.MF_EXX] = mag * np.cos(ang)
        marks[abi.MF_EXY] = mag * np.sin(ang)
    else:
        eta = 10.0 ** rng.uniform(20.0, 22.0, n)
        marks[abi.MF_EXX] = mexx * (1 + 0.05 * rng.normal(size=n))
        marks[abi.MF_EXY] = mexy * (1 + 0.05 * rng.normal(size=n))
        marks[abi.MF_XX] = 2 * eta * marks[abi.MF_EXX] + rng.normal(0, 1e5, n)
        marks[abi.MF_XY] = 2 * eta * marks[abi.MF_EXY] + rng.normal(0, 1e5, n)
    marks[abi.MF_P] = 3000.0 * 9.81 * (y + oy) + rng.normal(0, 1e5, n)
    marks[abi.MF_E] = np.abs(rng.normal(0, 0.01, n))
    marks[abi.MF_VX] = mvx * (1 + 0.01 * rng.normal(size=n))
    marks[abi.MF_VY] = mvy * (1 + 0.01 * rng.normal(size=n))
    marks[abi.MF_C] = np.zeros(n)
    r = np.abs(y + oy - 10e3)
    marks[abi.MF_PHI] = np.where(r <= 250.0, 8.0, 10.0) + 0.1 * rng.normal(size=n)
    marks[abi.MF_SLIPV] = 10.0 ** rng.uniform(-12, -8, n)
    for f in (abi.MF_D, abi.MF_W, abi.MF_V, abi.MF_C0, abi.MF_FRIC_STATIC,
              abi.MF_A, abi.MF_B, abi.MF_L, abi.MF_L0, abi.MF_V0):
        marks[f] = np.zeros(n)
    marks[abi.MF_D][:] = 2900.0

    # node fields (positions of the staggered unknowns)
    I, J = np.meshgrid(np.arange(xn), np.arange(yn), indexing="ij")
    I, J = I.ravel(), J.ravel()
    xb, yb = gx[I], gy[J]                                   # basic nodes
    Jp = np.minimum(J + 1, yn - 1)
    Ip = np.minimum(I + 1, xn - 1)
    xvx, yvx = gx[I], 0.5 * (gy[J] + gy[Jp])                # vx nodes
    xvy, yvy = 0.5 * (gx[I] + gx[Ip]), gy[J]                # vy nodes
    Im, Jm = np.maximum(I - 1, 0), np.maximum(J - 1, 0)
    xc, yc = 0.5 * (gx[Im] + gx[I]), 0.5 * (gy[Jm] + gy[J])  # pressure nodes
    nodes = {f: np.zeros(nn) for f in range(abi.NF_N)}

    def smooth(shape_scale, base):
        return base * (1 + shape_scale * rng.normal(size=nn))

    vx_, _, _, _, _ = _stream(xvx + ox, yvx + oy, XS, YS)
    _, vy_, _, _, _ = _stream(xvy + ox, yvy + oy, XS, YS)
    _, _, exx_c, _, _ = _stream(xc + ox, yc + oy, XS, YS)
    _, _, _, exy_b, esp_b = _stream(xb + ox, yb + oy, XS, YS)
    nodes[abi.NF_VX] = vx_
    nodes[abi.NF_VY] = vy_
    nodes[abi.NF_MVX] = vx_ * (1 + 1e-3 * rng.normal(size=nn))
    nodes[abi.NF_MVY] = vy_ * (1 + 1e-3 * rng.normal(size=nn))
    nodes[abi.NF_MVXE] = vx_ * (1 + 1e-3 * rng.normal(size=nn))
    nodes[abi.NF_MVYE] = vy_ * (1 + 1e-3 * rng.normal(size=nn))
    nodes[abi.NF_EXX] = exx_c
    nodes[abi.NF_EXXE] = exx_c * (1 + 1e-2 * rng.normal(size=nn))
    nodes[abi.NF_EXXEE] = exx_c * (1 + 1e-2 * rng.normal(size=nn))
    nodes[abi.NF_EXY] = exy_b
    nodes[abi.NF_EXYE] = exy_b * (1 + 1e-2 * rng.normal(size=nn))
    nodes[abi.NF_EXYEE] = exy_b * (1 + 1e-2 * rng.normal(size=nn))
    nodes[abi.NF_ESP] = esp_b
    eta_n = 1e21
    nodes[abi.NF_SXX] = 2 * eta_n * exx_c + rng.normal(0, 1e4, nn)
    nodes[abi.NF_SXXE] = nodes[abi.NF_SXX] * (1 + 1e-2 * rng.normal(size=nn))
    nodes[abi.NF_SXXEE] = nodes[abi.NF_SXX] * (1 + 1e-2 * rng.normal(size=nn))
    nodes[abi.NF_SXY] = 2 * eta_n * exy_b + rng.normal(0, 1e4, nn)
    nodes[abi.NF_SXYE] = nodes[abi.NF_SXY] * (1 + 1e-2 * rng.normal(size=nn))
    nodes[abi.NF_SXYEE] = nodes[abi.NF_SXY] * (1 + 1e-2 * rng.normal(size=nn))
    nodes[abi.NF_SXXS] = nodes[abi.NF_SXX] * (1 + 1e-2 * rng.normal(size=nn))
    nodes[abi.NF_PR] = 3000.0 * 9.81 * (yc + oy) + 10e6 + rng.normal(0, 1e4, nn)
    nodes[abi.NF_SPPE] = nodes[abi.NF_PR] * (1 + 1e-4 * rng.normal(size=nn))
    nodes[abi.NF_SPPEE] = nodes[abi.NF_PR] * (1 + 1e-4 * rng.normal(size=nn))
    nodes[abi.NF_SPPES] = nodes[abi.NF_PR] * (1 + 1e-4 * rng.normal(size=nn))
    ph = np.where(np.abs(yb + oy - 10e3) <= 100.0, 8.0, 50.0)
    nodes[abi.NF_PHIS] = ph + 0.05 * rng.normal(size=nn)
    nodes[abi.NF_PHIS_IT] = ph + 0.05 * rng.normal(size=nn)
    nodes[abi.NF_PHIE] = ph + 0.05 * rng.normal(size=nn)
    nodes[abi.NF_PE] = np.abs(rng.normal(0, 0.01, nn))
    nodes[abi.NF_PES] = nodes[abi.NF_PE] + 1e-4
    nodes[abi.NF_PEE] = nodes[abi.NF_PE] * (1 + 1e-2 * rng.normal(size=nn))
    nodes[abi.NF_RK_SLIPRS_FINAL] = 10.0 ** rng.uniform(-11, -8, nn)
    nodes[abi.NF_RK_PHIDTS_FINAL] = rng.normal(0, 1e-9, nn)
    nodes[abi.NF_RK_SLIPRS_SOLVED] = nodes[abi.NF_RK_SLIPRS_FINAL] * 1.1
    nodes[abi.NF_RK_PHIDTS_SOLVED] = nodes[abi.NF_RK_PHIDTS_FINAL] * 0.9
    nodes[abi.NF_EXXPL] = exx_c * 1e-2
    nodes[abi.NF_NU_M2C] = 10.0 ** rng.uniform(20, 23, nn)
    nodes[abi.NF_NU] = nodes[abi.NF_NU_M2C].copy()
    nodes[abi.NF_GG] = np.full(nn, 3.0e10)
    nodes[abi.NF_TK] = _temperature(yb + oy, YS)
    # fields the adaptive time step reads (calc_RSF.c:352-572): pressure at
    # basic nodes, bulk modulus, nodal friction parameters with the
    # velocity-weakening band, sticky-air flags, some very stiff nodes
    nodes[abi.NF_PRS] = 3000.0 * 9.81 * (yb + oy) + 10e6 + rng.normal(0, 1e4, nn)
    nodes[abi.NF_BM] = 5.0e10 * (1 + 0.1 * rng.uniform(size=nn))
    band = np.abs(yb + oy - 10e3) <= 100.0
    nodes[abi.NF_AS] = np.where(band, p["a_vw"], p["a_hr"]) * (1 + 0.01 * rng.uniform(size=nn))
    nodes[abi.NF_BS] = np.where(band, p["b_vw"], p["b_hr"]) * (1 + 0.01 * rng.uniform(size=nn))
    nodes[abi.NF_LS] = np.where(band, p["L_vw"], p["L_hr"]) * (1 + 0.01 * rng.uniform(size=nn))
    nodes[abi.NF_V0S] = np.where(band, p["V0_vw"], p["V0_hr"])
    nodes[abi.NF_STICKY01] = rng.choice([0.0, 1.0, 2.0], size=nn, p=[0.6, 0.3, 0.1])
    stiff = rng.uniform(size=nn) < 0.2
    nodes[abi.NF_NU_M2C][stiff] = 10.0 ** rng.uniform(26, 27, int(stiff.sum()))
    nodes[abi.NF_NU][stiff] = nodes[abi.NF_NU_M2C][stiff] * 0.5
    bondm, bondn, bondv = _bonds(xn, yn)
    return Case(name, p, gx, gy, rt, nodes, marks, t, bondm, bondn, bondv)

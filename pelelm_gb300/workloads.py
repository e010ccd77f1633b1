"""Seeded synthetic reactor inputs (no dataset exists for this path).

The state distribution follows the benchmark definitions: equivalence ratio phi and
progress variable c per cell; Y is a linear blend of the unburnt fuel-air mixture and its
complete-combustion products at that phi, plus 1e-6 of the H, O and OH radicals,
renormalised; T = T0 + c * U[a, b]; p fixed (or drawn); rho from the ideal-gas law;
rho h = rho * h(T, Y). Forcing (when requested) is N(0, sigma_Y^2) on rhoY projected to
zero sum over species and N(0, sigma_h^2) on rho h, drawn in MKS and converted to the
reactor's CGS units exactly as ``Source/PeleLM.cpp:5736-5746`` does (x1e-3, x10).

Cells are grouped into AMR-like boxes; each box owns one component-major block per field
(the FArrayBox/Array4 layout the reference's reactor receives: i fastest, then j, k, then
component).
"""
from __future__ import annotations

import copy
import functools
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from .mech.model import Mechanism, R_ERG, P_ATM

DATA_DIR = os.path.join(os.path.dirname(__file__), "data")


@functools.lru_cache(maxsize=None)
def _load_mechanism_cached(name: str) -> Mechanism:
    return Mechanism.from_json(os.path.join(DATA_DIR, f"{name}.json"))


def load_mechanism(name: str) -> Mechanism:
    """The named mechanism (a private copy: callers may modify it)."""
    return copy.deepcopy(_load_mechanism_cached(name))


def mech_path(name: str, ext: str = "mech") -> str:
    return os.path.join(DATA_DIR, f"{name}.{ext}")


# ------------------------------------------------------------------ thermo (numpy)
def _coeffs(mech: Mechanism):
    lo = np.array([s.low for s in mech.species])
    hi = np.array([s.high for s in mech.species])
    tm = np.array([s.Tmid for s in mech.species])
    W = np.array([s.W for s in mech.species])
    return lo, hi, tm, W


def species_h_mass(mech: Mechanism, T: np.ndarray) -> np.ndarray:
    """h_k(T) [erg/g], shape (ncell, ns)."""
    lo, hi, tm, W = _coeffs(mech)
    T = np.asarray(T, dtype=float)[:, None]

    def hRT(a):
        return (a[None, :, 0] + a[None, :, 1] * T / 2 + a[None, :, 2] * T ** 2 / 3 + a[None, :, 3] * T ** 3 / 4
                + a[None, :, 4] * T ** 4 / 5 + a[None, :, 5] / T)

    h = np.where(T < tm[None, :], hRT(lo), hRT(hi))
    return h * R_ERG * T / W[None, :]


def mixture_h(mech: Mechanism, T: np.ndarray, Y: np.ndarray) -> np.ndarray:
    return np.sum(species_h_mass(mech, T) * Y, axis=1)


# ------------------------------------------------------------------ compositions
def _mass_fractions(mech: Mechanism, moles: Dict[str, np.ndarray], n: int) -> np.ndarray:
    W = np.array([s.W for s in mech.species])
    X = np.zeros((n, mech.ns))
    for sname, x in moles.items():
        X[:, mech.index(sname)] += x
    m = X * W[None, :]
    return m / m.sum(axis=1, keepdims=True)


def h2_air(mech: Mechanism, phi: np.ndarray):
    n = phi.size
    unburnt = _mass_fractions(mech, {"H2": phi, "O2": 0.5 * np.ones(n), "N2": 1.88 * np.ones(n)}, n)
    water = np.minimum(phi, 1.0)
    burnt = _mass_fractions(mech, {"H2O": water, "H2": phi - water, "O2": 0.5 - 0.5 * water,
                                   "N2": 1.88 * np.ones(n)}, n)
    return unburnt, burnt


def ch4_air(mech: Mechanism, phi: np.ndarray):
    n = phi.size
    unburnt = _mass_fractions(mech, {"CH4": phi, "O2": 2.0 * np.ones(n), "N2": 7.52 * np.ones(n)}, n)
    burned = np.minimum(phi, 1.0)
    burnt = _mass_fractions(mech, {"CO2": burned, "H2O": 2 * burned, "CH4": phi - burned,
                                   "O2": 2.0 - 2.0 * burned, "N2": 7.52 * np.ones(n)}, n)
    return unburnt, burnt


# ------------------------------------------------------------------ configs
@dataclass
class Config:
    name: str
    mech: str
    boxes: List[int]                 # box side lengths (cubes)
    dt: float
    rtol: float = 1e-6
    atol: float = 1e-10
    phi: tuple = (0.5, 2.0)
    T0: float = 300.0
    dT: tuple = (900.0, 2100.0)      # T = T0 + c * U[dT]
    p_atm: tuple = (1.0, 1.0)
    forcing: bool = False
    sigma_Y_mks: float = 1e2         # kg/m^3/s
    sigma_h_mks: float = 1e8         # W/m^3
    fuel: str = "H2"
    description: str = ""

    @property
    def ncell(self) -> int:
        return int(sum(b ** 3 for b in self.boxes))


def _amr_boxes_cfg1() -> List[int]:
    # 120 boxes with sides from {8,16,32,64}: 6x64^3 + 14x32^3 + 20x16^3 + 80x8^3 = 2,154,496
    sides = [64] * 6 + [32] * 14 + [16] * 20 + [8] * 80
    rng = np.random.default_rng(1001)
    return [int(s) for s in rng.permutation(sides)]


def _boxes_cfg2() -> List[int]:
    sides = [32] * 48 + [16] * 128  # 2^21 cells
    rng = np.random.default_rng(1002)
    return [int(s) for s in rng.permutation(sides)]


def _boxes_cfg3() -> List[int]:
    sides = [32] * 96 + [16] * 256  # 2^22 cells
    rng = np.random.default_rng(1003)
    return [int(s) for s in rng.permutation(sides)]


def _boxes_cfg4() -> List[int]:
    sides = [64] * 2 + [32] * 14 + [16] * 14 + [8] * 16  # 2^20 cells
    rng = np.random.default_rng(1004)
    return [int(s) for s in rng.permutation(sides)]


CONFIGS: Dict[str, Config] = {
    "lidryer_32cube": Config(
        "lidryer_32cube", "lidryer_syn", [32], dt=1e-6,
        description="LiDryer-shaped H2/O2 (9 sp, 21 rx), 32^3 = 32768 cells in one box, "
                    "dt_react 1e-6 s, rtol 1e-6, atol 1e-10, zero forcing"),
    "lidryer_amr120": Config(
        "lidryer_amr120", "lidryer_syn", _amr_boxes_cfg1(), dt=1e-5, forcing=True,
        description="LiDryer-shaped H2/O2, 120 boxes {8,16,32,64}^3 = 2,154,496 cells, "
                    "dt_react 1e-5 s, N(0,1e2^2) kg/m^3/s species and N(0,1e8^2) W/m^3 "
                    "energy forcing"),
    "drm19_2M": Config(
        "drm19_2M", "drm19_syn", _boxes_cfg2(), dt=1e-5, forcing=True, fuel="CH4",
        phi=(0.6, 1.4), dT=(1900.0, 1900.0),
        description="drm19-shaped CH4/air (21 sp, 84 rx), 2^21 cells in 16^3/32^3 boxes, "
                    "dt_react 1e-5 s, forcing as lidryer_amr120"),
    "drm19_4M": Config(
        "drm19_4M", "drm19_syn", _boxes_cfg3(), dt=1e-5, forcing=True, fuel="CH4",
        phi=(0.6, 1.4), dT=(1900.0, 1900.0),
        description="drm19-shaped CH4/air, the drm19_2M state distribution on 2^22 cells in "
                    "16^3/32^3 boxes (surrogate inference workload)"),
    "gri_1M": Config(
        "gri_1M", "gri_syn", _boxes_cfg4(), dt=1e-5, forcing=True, fuel="CH4",
        phi=(0.5, 1.5), dT=(2100.0, 2100.0), p_atm=(1.0, 10.0),
        description="GRI-shaped CH4/air (53 sp, 325 rx), 2^20 cells in 8^3-64^3 boxes, "
                    "p ~ U[1,10] atm, dt_react 1e-5 s"),
}


@dataclass
class CellState:
    """Flat per-cell state (cell-major views convenient for tests), CGS units."""
    rY: np.ndarray       # (ncell, ns) g/cm^3
    rYsrc: np.ndarray    # (ncell, ns) g/cm^3/s
    T: np.ndarray        # (ncell,)
    rE: np.ndarray       # (ncell,) erg/cm^3
    rEsrc: np.ndarray    # (ncell,) erg/cm^3/s
    mask: np.ndarray     # (ncell,) int32
    p: np.ndarray        # (ncell,) dyn/cm^2

    @property
    def ncell(self) -> int:
        return self.T.size


def make_cells(cfg: Config, ncell: Optional[int] = None, seed: int = 0) -> CellState:
    mech = _load_mechanism_cached(cfg.mech)  # read only
    n = cfg.ncell if ncell is None else int(ncell)
    rng = np.random.default_rng(seed)
    phi = rng.uniform(cfg.phi[0], cfg.phi[1], n)
    c = rng.uniform(0.0, 1.0, n)
    if cfg.fuel == "H2":
        Yu, Yb = h2_air(mech, phi)
    else:
        Yu, Yb = ch4_air(mech, phi)
    Y = (1.0 - c)[:, None] * Yu + c[:, None] * Yb
    for r in ("H", "O", "OH"):
        Y[:, mech.index(r)] += 1e-6
    Y /= Y.sum(axis=1, keepdims=True)
    T = cfg.T0 + c * rng.uniform(cfg.dT[0], cfg.dT[1], n)
    p = P_ATM * rng.uniform(cfg.p_atm[0], cfg.p_atm[1], n)
    W = np.array([s.W for s in mech.species])
    Wbar = 1.0 / np.sum(Y / W[None, :], axis=1)
    rho = p * Wbar / (R_ERG * T)
    rY = rho[:, None] * Y
    rE = rho * mixture_h(mech, T, Y)
    rYsrc = np.zeros_like(rY)
    rEsrc = np.zeros(n)
    if cfg.forcing:
        f = rng.normal(0.0, cfg.sigma_Y_mks, (n, mech.ns)) * 1e-3  # kg/m^3/s -> g/cm^3/s
        # Realizability: transport cannot remove more of a species than a cell holds, so the
        # forcing alone may drain at most half of each species over dt_react ...
        f = np.maximum(f, -0.5 * rY / cfg.dt)
        # ... then project to zero net mass source along Y (keeps every bound above).
        f -= f.sum(axis=1, keepdims=True) * Y
        rYsrc = f
        rEsrc = rng.normal(0.0, cfg.sigma_h_mks, n) * 10.0  # W/m^3 -> erg/cm^3/s
    mask = np.ones(n, dtype=np.int32)
    return CellState(rY=rY, rYsrc=rYsrc, T=T, rE=rE, rEsrc=rEsrc, mask=mask, p=p)


def make_box_cells(cfg: Config, sides: List[int], box_ids, seed: int = 0) -> CellState:
    """Cells of the cubic boxes `box_ids` of a box list with sides `sides` (cells of one box in
    i-fastest order, boxes in the order given). Box b draws from its own stream, seeded
    (seed, b), so any subset of a box list, on any rank, gets the same cells as the whole."""
    parts = [make_cells(cfg, int(sides[b]) ** 3, seed=[int(seed), int(b)]) for b in box_ids]
    if not parts:
        return make_cells(cfg, 0, seed=seed)
    return CellState(**{k: np.concatenate([getattr(p, k) for p in parts]) for k in CellState.__annotations__})


@dataclass
class BoxLayout:
    """Boxes of a config packed into one arena per field (component-major per box)."""
    sides: List[int]
    cell_offset: np.ndarray   # (nbox+1,) first cell of each box in flat cell order

    @property
    def nbox(self) -> int:
        return len(self.sides)

    @property
    def ncell(self) -> int:
        return int(self.cell_offset[-1])


def box_layout(sides: List[int]) -> BoxLayout:
    off = np.zeros(len(sides) + 1, dtype=np.int64)
    off[1:] = np.cumsum([s ** 3 for s in sides])
    return BoxLayout(sides=list(sides), cell_offset=off)


def to_box_arena(layout: BoxLayout, a: np.ndarray) -> np.ndarray:
    """(ncell, ncomp) cell-major -> arena where box b holds a [ncomp][cells_b] block."""
    a2 = a if a.ndim == 2 else a[:, None]
    ncomp = a2.shape[1]
    out = np.empty(layout.ncell * ncomp, dtype=a2.dtype)
    for b in range(layout.nbox):
        c0, c1 = layout.cell_offset[b], layout.cell_offset[b + 1]
        out[c0 * ncomp:c1 * ncomp] = a2[c0:c1].T.reshape(-1)
    return out


def from_box_arena(layout: BoxLayout, arena: np.ndarray, ncomp: int) -> np.ndarray:
    out = np.empty((layout.ncell, ncomp), dtype=arena.dtype)
    for b in range(layout.nbox):
        c0, c1 = layout.cell_offset[b], layout.cell_offset[b + 1]
        out[c0:c1] = arena[c0 * ncomp:c1 * ncomp].reshape(ncomp, c1 - c0).T
    return out if ncomp > 1 else out[:, 0]


def typical_atol(cfg: Config, ns: int) -> np.ndarray:
    """Uniform absolute tolerance on the CGS ODE vector [rhoY_1..rhoY_ns, T]."""
    return np.full(ns + 1, cfg.atol)

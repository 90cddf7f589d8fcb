"""Seeded synthetic gases for the electron Monte Carlo path, and their LXCat form.

The reference ships no benchmark gases for its headline workloads, so the
workloads are generated here from a seed:

* ``atomic_gas``   - one atom, constant elastic 6e-20 m^2 plus one excitation
  at 11.5 eV rising linearly to 2e-21 m^2 at 30 eV (100 log points).
* ``n2_like_gas``  - elastic (screened-Coulomb anisotropy), one rotational
  ``<->`` level at 0.0012 eV, 8 vibrational ``<->`` levels (0.29-2.3 eV),
  20 electronic levels (6-15 eV) and one ionization (15.6 eV), every cross
  section a smooth seeded bump with peak 1e-22..1e-19 m^2 on 200 log points.
* ``o2_like_gas``  - 25 processes including dissociative attachment at 4.4 eV
  (peak 1.4e-22 m^2).
* ``random_gas``   - 10-40 processes on 100-400 point grids (request streams).

Each gas is a list of LXCat-style collisions. ``flatten`` turns a mixture into
the per-process arrays the engine consumes, following the reference's own
flattening (Code/LoKI-MC/Sources/BoltzmannMC.C:29-271 and the Collision
constructor, Code/LoKI-MC/Sources/Collision.C:18-45). ``write_lxcat`` and
``write_setup`` emit the same mixture as reference input files
(LXCat grammar of Code/LoKI-MC/Sources/Parse.C:43-295, setup keys of
Code/LoKI-MC/Headers/BoltzmannMC.h:262-376) for the parity fixtures.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import constants as C

KB_EV = C.BOLTZMANN / C.ELECTRON_CHARGE


@dataclass
class Collision:
    ctype: str                 # Elastic, Excitation, Vibrational, Rotational, Ionization, Attachment, Effective
    target: str                # state name, e.g. "X2(X,v=0)"
    product: str               # state name (same as target for Elastic)
    threshold: float           # eV (0 for Elastic)
    energies: np.ndarray       # raw LXCat energies (eV)
    values: np.ndarray         # raw LXCat integral cross sections (m^2)
    reverse: bool = False      # "<->": adds a superelastic process
    sampler: str = "isotropic"
    sampler_params: Sequence[float] = ()


@dataclass
class State:
    population: float
    weight: float = 1.0
    energy: float = 0.0


@dataclass
class Gas:
    name: str
    mass: float                       # kg
    fraction: float
    collisions: List[Collision]
    states: Dict[str, State]
    opb: Optional[float] = None       # OPB parameter (eV) for SDCS sharing; None -> threshold

    def density(self, state: str) -> float:
        """Relative density of a state: product of populations along its
        ele/vib/rot hierarchy times the gas fraction
        (Code/LoKI-MC/Headers/State.h:72-85)."""
        inner = state[state.index("(") + 1:state.rindex(")")]
        parts = inner.split(",")
        base = state[:state.index("(")]
        d = self.fraction
        for k in range(1, len(parts) + 1):
            name = f"{base}({','.join(parts[:k])})"
            d *= self.states[name].population
        return d


def log_grid(n: int, lo: float = 1e-3, hi: float = 1e3) -> np.ndarray:
    return np.logspace(math.log10(lo), math.log10(hi), n)


def _bump(e: np.ndarray, thr: float, peak: float, center: float, width: float, tail: float) -> np.ndarray:
    """Smooth resonance: zero below threshold, log-Gaussian bump at ``center``
    with relative ``width`` plus a slowly decaying tail; max equals ``peak``."""
    x = np.where(e > thr, e, thr)
    g = np.exp(-0.5 * (np.log(x / center) / width) ** 2)
    t = tail * np.sqrt(np.maximum(x - thr, 0.0) / (x - thr + center))
    s = g + t
    s = np.where(e > thr, s, 0.0)
    m = s.max()
    return peak * s / m if m > 0 else s


def atomic_gas(name: str = "A1") -> Gas:
    """Single synthetic atom: N=3.22e22, T=300 K, m/M=1.37e-4; constant elastic
    6e-20 m^2 (isotropic); excitation at 11.5 eV, linear to 2e-21 m^2 at 30 eV,
    then flat; both on 100 log points over 1e-3..1e3 eV."""
    e = log_grid(100)
    el = Collision("Elastic", f"{name}(gnd)", f"{name}(gnd)", 0.0, e, np.full_like(e, 6e-20))
    exc_v = np.where(e < 11.5, 0.0, np.where(e < 30.0, 2e-21 * (e - 11.5) / (30.0 - 11.5), 2e-21))
    ex = Collision("Excitation", f"{name}(gnd)", f"{name}(exc)", 11.5, e, exc_v)
    return Gas(name, C.ELECTRON_MASS / 1.37e-4, 1.0, [el, ex],
               {f"{name}(gnd)": State(1.0), f"{name}(exc)": State(0.0)})


def maxwell_gas(nu: float, density: float, name: str = "M1", mass_ratio: float = 1.37e-4) -> Gas:
    """Maxwell-model gas: elastic cross section nu/(N*sqrt(2 e eps/m)) so that
    the momentum-transfer frequency is constant (nu, s^-1), isotropic."""
    e = log_grid(400, 1e-4, 1e3)
    v = np.sqrt(2.0 * e * C.ELECTRON_CHARGE / C.ELECTRON_MASS)
    sig = nu / (density * v)
    el = Collision("Elastic", f"{name}(gnd)", f"{name}(gnd)", 0.0, e, sig)
    return Gas(name, C.ELECTRON_MASS / mass_ratio, 1.0, [el], {f"{name}(gnd)": State(1.0)})


def reid_ramp_gas(name: str = "A") -> Gas:
    """Reid's ramp model gas (Reid 1979, Aust. J. Phys. 32, 231), the
    reference's benchmark case 1: target mass 4 amu, constant isotropic elastic
    cross section 6e-20 m^2, one excitation with threshold 0.2 eV and cross
    section 1e-19 (eps - 0.2) m^2 (eps in eV), each tabulated at its two end
    points (linear between them) up to 1000 eV."""
    mass = 4.0 * 1.660539040e-27
    el = Collision("Elastic", f"{name}(gnd)", f"{name}(gnd)", 0.0, np.array([0.0, 1000.0]),
                   np.array([6e-20, 6e-20]))
    ex = Collision("Excitation", f"{name}(gnd)", f"{name}(exc)", 0.2, np.array([0.2, 1000.0]),
                   np.array([0.0, 1e-19 * (1000.0 - 0.2)]))
    return Gas(name, mass, 1.0, [el, ex], {f"{name}(gnd)": State(1.0), f"{name}(exc)": State(0.0)})


def _boltzmann(energies: Sequence[float], weights: Sequence[float], tg: float) -> List[float]:
    z = [w * math.exp(-en / (KB_EV * tg)) for en, w in zip(energies, weights)]
    s = sum(z)
    return [v / s for v in z]


def molecular_gas(name: str, seed: int, *, mass_amu: float, n_vib: int, vib_lo: float, vib_hi: float,
                  n_ele: int, ele_lo: float, ele_hi: float, ion_thr: Optional[float],
                  rot_thr: Optional[float], att: Optional[tuple], n_points: int = 200,
                  screen: bool = True, tg: float = 300.0, fraction: float = 1.0, e_max: float = 1e3) -> Gas:
    """Seeded molecule with elastic, rotational/vibrational ``<->`` levels,
    electronic levels, optional ionization and attachment; cross sections on
    ``n_points`` log points over 1e-3..``e_max`` eV (the same seeded shapes for
    any ``e_max``)."""
    rng = np.random.default_rng(seed)
    e = log_grid(n_points, 1e-3, e_max)
    cols: List[Collision] = []
    states: Dict[str, State] = {f"{name}(X)": State(1.0, 1.0, 0.0)}
    ground = f"{name}(X)"
    v0 = f"{name}(X,v=0)"

    # elastic (integral) with a screened-Coulomb anisotropy
    el_peak = 10 ** rng.uniform(-19.5, -19.0)
    el = 0.45 * el_peak + _bump(e, 0.0, 0.55 * el_peak, 10 ** rng.uniform(0.0, 1.0), 0.8, 0.0)
    el = np.where(e > 0, el, el)
    sampler = "coulombScreen" if screen else "isotropic"
    params = (0.0, float(np.round(10 ** rng.uniform(-0.5, 0.5), 6))) if screen else ()
    cols.append(Collision("Elastic", ground, ground, 0.0, e, el, sampler=sampler, sampler_params=params))

    vib_thr = list(np.round(np.linspace(vib_lo, vib_hi, n_vib), 6)) if n_vib else []
    vib_names = [f"{name}(X,v={k})" for k in range(n_vib + 1)]
    vib_pop = _boltzmann([0.0] + vib_thr, [1.0] * (n_vib + 1), tg)
    for k, vn in enumerate(vib_names):
        states[vn] = State(vib_pop[k], 1.0, ([0.0] + vib_thr)[k])

    if rot_thr is not None:
        j0, j2 = f"{name}(X,v=0,J=0)", f"{name}(X,v=0,J=2)"
        rp = _boltzmann([0.0, rot_thr], [1.0, 5.0], tg)
        states[j0] = State(rp[0], 1.0, 0.0)
        states[j2] = State(rp[1], 5.0, rot_thr)
        peak = 10 ** rng.uniform(-21.0, -20.0)
        sig = _bump(e, rot_thr, peak, 10 ** rng.uniform(-1.5, -0.5), 1.2, 0.3)
        cols.append(Collision("Rotational", j0, j2, float(rot_thr), e, sig, reverse=True))

    for k, thr in enumerate(vib_thr, start=1):
        peak = 10 ** rng.uniform(-21.5, -19.7)
        ctr = max(thr * 1.2, 10 ** rng.uniform(0.2, 0.6))
        sig = _bump(e, thr, peak, ctr, 0.25, 0.02)
        cols.append(Collision("Vibrational", v0, vib_names[k], float(thr), e, sig, reverse=True))

    if att is not None:
        thr, peak = att
        sig = _bump(e, thr, peak, thr * 1.5, 0.15, 0.0)
        cols.append(Collision("Attachment", ground, f"{name}(-)", float(thr), e, sig))
        states[f"{name}(-)"] = State(0.0)

    ele_thr = list(np.round(np.linspace(ele_lo, ele_hi, n_ele), 6)) if n_ele else []
    for k, thr in enumerate(ele_thr):
        peak = 10 ** rng.uniform(-22.0, -20.3)
        ctr = thr * 10 ** rng.uniform(0.15, 0.6)
        sig = _bump(e, thr, peak, ctr, 0.6, 0.4)
        st = f"{name}(E{k + 1})"
        states[st] = State(0.0)
        cols.append(Collision("Excitation", ground, st, float(thr), e, sig))

    if ion_thr is not None:
        peak = 10 ** rng.uniform(-20.0, -19.4)
        sig = _bump(e, ion_thr, peak, ion_thr * 6.0, 0.9, 0.3)
        cols.append(Collision("Ionization", ground, f"{name}(+)", float(ion_thr), e, sig))
        states[f"{name}(+)"] = State(0.0)

    return Gas(name, mass_amu * C.UNIFIED_ATOMIC_MASS, fraction, cols, states)


def n2_like_gas(seed: int = 2, name: str = "X2", fraction: float = 1.0, e_max: float = 1e3) -> Gas:
    return molecular_gas(name, seed, mass_amu=28.0, n_vib=8, vib_lo=0.29, vib_hi=2.3, n_ele=20,
                         ele_lo=6.0, ele_hi=15.0, ion_thr=15.6, rot_thr=0.0012, att=None,
                         fraction=fraction, e_max=e_max)


def o2_like_gas(seed: int = 3, name: str = "Y2", fraction: float = 1.0, e_max: float = 1e3) -> Gas:
    # 1 elastic + 1 rot (<->: 2) + 4 vib (<->: 8) + 1 attachment + 12 electronic + 1 ionization = 25
    return molecular_gas(name, seed, mass_amu=32.0, n_vib=4, vib_lo=0.19, vib_hi=0.75, n_ele=12,
                         ele_lo=0.98, ele_hi=14.0, ion_thr=12.07, rot_thr=0.0018,
                         att=(4.4, 1.4e-22), fraction=fraction, e_max=e_max)


def random_gas(seed: int, name: str, fraction: float, e_max: float = 1e3) -> Gas:
    """Request-stream gas: 10-40 processes on a 100-400 point grid."""
    rng = np.random.default_rng(seed)
    n_pts = int(rng.integers(100, 401))
    n_target = int(rng.integers(10, 41))
    n_vib = int(rng.integers(0, min(8, (n_target - 3) // 2) + 1))
    n_ele = max(1, n_target - 1 - 2 - 2 * n_vib - 2)
    att = (float(np.round(rng.uniform(3.0, 6.0), 3)), float(10 ** rng.uniform(-22.5, -21.5))) \
        if rng.random() < 0.5 else None
    return molecular_gas(name, seed, mass_amu=float(rng.uniform(14.0, 44.0)), n_vib=n_vib,
                         vib_lo=0.15, vib_hi=0.15 + 0.3 * max(n_vib, 1), n_ele=n_ele,
                         ele_lo=float(rng.uniform(5.0, 8.0)), ele_hi=float(rng.uniform(10.0, 16.0)),
                         ion_thr=float(rng.uniform(12.0, 16.0)), rot_thr=0.002, att=att,
                         n_points=n_pts, fraction=fraction, e_max=e_max)


# ---------------------------------------------------------------------------
# Flattening: mixture -> per-process arrays
# ---------------------------------------------------------------------------

@dataclass
class ProcessSet:
    """Per-process arrays in the order the reference builds them
    (BoltzmannMC.C:29-271): every non-Effective collision once, followed by
    its superelastic copy when it is reversible."""
    ptype: np.ndarray        # int32: 0 conservative, 1 ionization, 2 attachment
    is_super: np.ndarray     # int32
    is_elastic: np.ndarray   # int32 (power bookkeeping only)
    sampler: np.ndarray      # int32 sampler code
    sampler_p0: np.ndarray
    sampler_p1: np.ndarray
    superw: np.ndarray       # g_target / g_product for superelastic, else 0
    emin: np.ndarray         # threshold (inelastic) or 0 (superelastic)
    emax: np.ndarray         # last raw energy (inelastic) or emax[p-1] - threshold
    rel_dens: np.ndarray
    mass: np.ndarray         # target mass, kg
    red_mass: np.ndarray
    eloss: np.ndarray        # threshold, negative for superelastic
    wparam: np.ndarray       # ionization w (OPB or threshold), else 0
    raw_e: List[np.ndarray]  # threshold-clipped raw energies (superelastic: [0])
    raw_v: List[np.ndarray]
    gas_first: np.ndarray    # first process index per gas with collisions
    gas_last: np.ndarray
    gas_fraction: np.ndarray
    energy_max_elastic: float
    ctype: List[str] = field(default_factory=list)   # collision type per process
    gas_index: np.ndarray = None                    # gas of each process
    descr: List[str] = field(default_factory=list)

    @property
    def n(self) -> int:
        return int(self.ptype.shape[0])


def _clip_raw(col: Collision):
    e = [float(x) for x in col.energies]
    v = [float(x) for x in col.values]
    if col.ctype in ("Elastic", "Effective") and e[0] != 0:
        # Collision.C:40-43: insert an eps=0 point with the first value
        e.insert(0, 0.0)
        v.insert(0, v[0])
    thr = col.threshold
    while e[0] < thr:            # BoltzmannMC.C:139-142
        e.pop(0)
        v.pop(0)
    if e[0] != thr:              # BoltzmannMC.C:144-147
        e.insert(0, thr)
        v.insert(0, 0.0)
    return np.array(e), np.array(v)


def flatten(gases: Sequence[Gas]) -> ProcessSet:
    me = C.ELECTRON_MASS
    rows = dict(ptype=[], is_super=[], is_elastic=[], sampler=[], sampler_p0=[], sampler_p1=[], superw=[],
                emin=[], emax=[], rel_dens=[], mass=[], red_mass=[], eloss=[], wparam=[])
    raw_e, raw_v, ctype, gidx, descr = [], [], [], [], []
    first, last, frac = [], [], []
    emax_el = 1e100
    it = 0
    for gi, gas in enumerate(gases):
        cols = [c for c in gas.collisions]
        if not cols:
            continue
        first.append(it)
        frac.append(gas.fraction)
        for col in cols:
            if col.ctype == "Effective":
                continue
            pt = {"Ionization": C.IONIZATION, "Attachment": C.ATTACHMENT}.get(col.ctype, C.CONSERVATIVE)
            e, v = _clip_raw(col)
            sc = C.SAMPLER_NAMES[col.sampler]
            p = list(col.sampler_params) + [0.0, 0.0]
            rows["ptype"].append(pt)
            rows["is_super"].append(0)
            rows["is_elastic"].append(1 if col.ctype == "Elastic" else 0)
            rows["sampler"].append(sc)
            rows["sampler_p0"].append(p[0])
            rows["sampler_p1"].append(p[1])
            rows["superw"].append(0.0)
            rows["emin"].append(col.threshold)
            rows["emax"].append(float(e[-1]))
            rows["rel_dens"].append(gas.density(col.target))
            rows["mass"].append(gas.mass)
            rows["red_mass"].append(me * gas.mass / (me + gas.mass))
            rows["eloss"].append(col.threshold)
            rows["wparam"].append((gas.opb if gas.opb is not None else col.threshold)
                                  if col.ctype == "Ionization" else 0.0)
            if col.ctype == "Elastic":
                emax_el = min(emax_el, float(e[-1]))
            raw_e.append(e)
            raw_v.append(v)
            ctype.append(col.ctype)
            gidx.append(gi)
            descr.append(f"e+{col.target}{'<->' if col.reverse else '->'}e+{col.product},{col.ctype}")
            it += 1
            if col.reverse:
                rows["ptype"].append(C.CONSERVATIVE)
                rows["is_super"].append(1)
                rows["is_elastic"].append(0)
                rows["sampler"].append(sc)
                rows["sampler_p0"].append(p[0])
                rows["sampler_p1"].append(p[1])
                rows["superw"].append(gas.states[col.target].weight / gas.states[col.product].weight)
                rows["emin"].append(0.0)
                rows["emax"].append(rows["emax"][-1] - col.threshold)
                rows["rel_dens"].append(gas.density(col.product))
                rows["mass"].append(gas.mass)
                rows["red_mass"].append(me * gas.mass / (me + gas.mass))
                rows["eloss"].append(-col.threshold)
                rows["wparam"].append(0.0)
                raw_e.append(np.zeros(1))
                raw_v.append(np.zeros(1))
                ctype.append(col.ctype)
                gidx.append(gi)
                descr.append(descr[-1] + "(super)")
                it += 1
        last.append(it - 1)
    ints = ("ptype", "is_super", "is_elastic", "sampler")
    arr = {k: np.array(v, dtype=np.int32 if k in ints else np.float64) for k, v in rows.items()}
    return ProcessSet(raw_e=raw_e, raw_v=raw_v, gas_first=np.array(first, np.int32),
                      gas_last=np.array(last, np.int32), gas_fraction=np.array(frac, np.float64),
                      energy_max_elastic=emax_el, ctype=ctype, gas_index=np.array(gidx, np.int32),
                      descr=descr, **arr)


# ---------------------------------------------------------------------------
# Reference input files
# ---------------------------------------------------------------------------

def _fmt(x: float) -> str:
    return repr(float(x))


def write_lxcat(gas: Gas, path: str) -> None:
    """One LXCat block per collision, in the grammar Parse.C:43-125 reads:
    PROCESS line, PARAM. line with ``E = x eV`` (not needed for Elastic),
    the bracketed description line, dashed-delimited two-column data."""
    out = []
    for col in gas.collisions:
        arrow = "<->" if col.reverse else "->"
        out.append(f"SPECIES: e / {gas.name}")
        out.append(f"PROCESS: E + {gas.name} -> E + {gas.name}, {col.ctype}")
        if col.ctype in ("Elastic", "Effective"):
            out.append(f"PARAM.:  m/M = {C.ELECTRON_MASS / gas.mass!r}")
            sub = ", Integral"
        else:
            out.append(f"PARAM.:  E = {_fmt(col.threshold)} eV")
            sub = ""
        prod = "" if col.ctype == "Attachment" else "e + "
        lhs = f"e + {col.target}"
        rhs = f"{prod}{col.product}" if col.ctype != "Ionization" else f"e + e + {col.product}"
        out.append(f"COMMENT: [{lhs} {arrow} {rhs}, {col.ctype}{sub}]")
        out.append("COLUMNS: Energy (eV) | Cross section (m2)")
        out.append("-----------------------------")
        for x, y in zip(col.energies, col.values):
            out.append(f"{_fmt(x)} {_fmt(y)}")
        out.append("-----------------------------")
        out.append("")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def write_setup(path: str, lxcat_files: Sequence[str], gases: Sequence[Gas], *, pressure_pa: float,
                tg: float = 300.0, red_field=100.0, red_mag=0.0, angle=180.0, freq=0.0,
                n_electrons: float = 1e4, sharing: str = "equalSharing", gas_temp: str = "false",
                extra_numerics: Optional[Dict[str, str]] = None, anis: Optional[List[str]] = None,
                folder: str = "out", output: bool = False, kte_init_ev: Optional[float] = None,
                data_files: Sequence[str] = ("eedf", "swarmParameters", "rateCoefficients", "powerBalance",
                                             "MCSimDetails"),
                n_phases: Optional[int] = None) -> None:
    """A reference setup file (.in) for the mixture, gui off."""
    def vec(v):
        if isinstance(v, (list, tuple, np.ndarray)):
            return "[" + ",".join(_fmt(x) for x in v) + "]"
        return _fmt(v)

    L = ["workingConditions:",
         f"  gasPressure: {_fmt(pressure_pa)}",
         f"  gasTemperature: {_fmt(tg)}",
         f"  reducedElecField: {vec(red_field)}",
         f"  reducedMagField: {vec(red_mag)}",
         f"  elecFieldAngle: {vec(angle)}",
         f"  excitationFrequency: {vec(freq)}",
         "electronKinetics:",
         "  isOn: true",
         "  eedfType: boltzmannMC",
         f"  ionizationOperatorType: {sharing}",
         "  LXCatFiles:"]
    L += [f"    - {f}" for f in lxcat_files]
    if anis:
        L += ["  anisotropicScattering:", "    isOn: true", "    angleNumber: 1000", "    collisions:"]
        L += [f"      - {a}" for a in anis]
    L += ["  gasProperties:", "    mass:"]
    L += [f"      - {g.name} = {_fmt(g.mass)}" for g in gases]
    L += ["    fraction:"]
    L += [f"      - {g.name} = {_fmt(g.fraction)}" for g in gases]
    if any(g.opb is not None for g in gases):
        L += ["    OPBParameter:"]
        L += [f"      - {g.name} = {_fmt(g.opb)}" for g in gases if g.opb is not None]
    L += ["  stateProperties:", "    energy:"]
    for g in gases:
        for s, st in g.states.items():
            L.append(f"      - {s} = {_fmt(st.energy)}")
    L += ["    statisticalWeight:"]
    for g in gases:
        for s, st in g.states.items():
            L.append(f"      - {s} = {_fmt(st.weight)}")
    L += ["    population:"]
    for g in gases:
        for s, st in g.states.items():
            L.append(f"      - {s} = {_fmt(st.population)}")
    L += ["  numericsMC:",
          f"    nElectrons: {_fmt(n_electrons)}",
          f"    gasTemperatureEffect: {gas_temp}"]
    if kte_init_ev is not None:
        L.append(f"    initialElecTempOverGasTemp: {_fmt(kte_init_ev / (KB_EV * tg))}")
    for k, v in (extra_numerics or {}).items():
        L.append(f"    {k}: {v}")
    if n_phases is not None:
        L.append(f"    nIntegrationPhases: {int(n_phases)}")
    L += ["gui:", "  isOn: false", "output:", f"  isOn: {'true' if output else 'false'}",
          f"  folder: {folder}", "  dataFiles:"]
    L += [f"    - {d}" for d in data_files]
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def anis_lines(gases: Sequence[Gas]) -> List[str]:
    """anisotropicScattering.collisions entries ("group;gas;type;law;params",
    Setup.h:351-459), one per (gas, collision type) with a non-isotropic law.
    A group line sets every collision of that type in the gas, so a gas keeps
    one law per collision type."""
    out, seen = [], set()
    for g in gases:
        for c in g.collisions:
            if c.sampler == "isotropic" or (g.name, c.ctype) in seen:
                continue
            seen.add((g.name, c.ctype))
            p = ",".join(_fmt(x) for x in c.sampler_params)
            out.append(f"group;{g.name};{c.ctype};{c.sampler};{p}" if p else
                       f"group;{g.name};{c.ctype};{c.sampler}")
    return out


def assign_sampler(gas: Gas, ctype: str, sampler: str, params: Sequence[float] = ()) -> Gas:
    """Sets the angular scattering law of every collision of one type."""
    for c in gas.collisions:
        if c.ctype == ctype:
            c.sampler = sampler
            c.sampler_params = tuple(params)
    return gas


def write_case(dirpath: str, gases: Sequence[Gas], setup_name: str = "case.in", **kw) -> str:
    """Writes Input/<gas>.txt for every gas plus Input/<setup_name>; returns
    the setup path relative to Input/."""
    inp = os.path.join(dirpath, "Input")
    os.makedirs(inp, exist_ok=True)
    files = []
    for g in gases:
        fn = f"{g.name}_LXCat.txt"
        write_lxcat(g, os.path.join(inp, fn))
        files.append(fn)
    anis = anis_lines(gases)
    write_setup(os.path.join(inp, setup_name), files, gases, anis=anis or None, **kw)
    return setup_name

"""Host-side mirror of exaStamp's operators for the MD hot path.

Each class keeps the reference operator's name, slot names, slot meaning and
error behaviour (a missing REQUIRED slot or an inconsistent species list
raises `OperatorError`, where the reference calls ``fatal_error()``), and
executes through the C ABI of libgbmd.so.  A run description is a plain dict
shaped like the reference's YAML (``.msp``) maps, for example::

    {"species": [{"Ar": {"mass": 39.948}}],
     "lj_compute_force": {"rcut": 8.0, "parameters": {"epsilon": 1.0, "sigma": 1.0}}}

Reference operators mirrored (paths in the exaStamp tree):
  lj_compute_force          src/potential/pair_potential_template/pair_potential_impl.hxx L104-121, L417-446
  lj_multi_force            src/potential/pair_potential_template/pair_potential_force_op_multiparam.h L249-284
  eam_alloy_force           src/potential/eam_potential_template/eam_potential_multimat.cu L88-109, L113-257
  zero_force_energy, force_to_accel   src/compute/zero_force_energy.cu, src/compute/force_to_accel.cu
  push_f_v_r / push_f_v     data/config/config_numerical_schemes.msp L23-28 (exaNBody operators)
  push_f_v_r_xform_minimization  src/numerical_schemes/push_vec3_2nd_order_xform_minimization.cpp L56-95
  chunk_neighbors           data/config/config_move_particles.msp L54-68 (exaNBody operator)
  simulation_thermodynamic_state  src/thermo_state/simulation_thermodynamic_state.cpp L57-238
"""
from __future__ import annotations

import re
from dataclasses import dataclass

import numpy as np

from . import _capi
from .setfl import Setfl, read_setfl
from .systems import EV

_UNIT = {  # to the reference's internal system: angstrom, dalton, picosecond
    "ang": 1.0, "angstrom": 1.0, "nm": 10.0, "m": 1e10,
    "eV": EV, "J": 1.0 / 1.66053906660e-23,
    "Da": 1.0, "dalton": 1.0, "ps": 1.0, "fs": 1e-3, "s": 1e12,
}


class OperatorError(RuntimeError):
    """Raised where the reference operator calls fatal_error() / std::abort()."""


def quantity(v) -> float:
    """'3.4 ang' / '0.0104 eV' / '3.08 eV/ang' / 2.5 -> float in internal units."""
    if isinstance(v, (int, float)):
        return float(v)
    m = re.fullmatch(r"\s*([-+0-9.eE]+)\s*([A-Za-z]*)\s*(?:/\s*([A-Za-z]+))?\s*", str(v))
    if not m:
        raise OperatorError("cannot parse quantity %r" % (v,))
    val, unit, per = float(m.group(1)), m.group(2), m.group(3)
    for u in (unit, per):
        if u and u not in _UNIT:
            raise OperatorError("unsupported unit %r" % u)
    f = _UNIT[unit] if unit else 1.0
    if per:
        f /= _UNIT[per]
    return val * f


@dataclass
class ThermodynamicState:
    """Derived quantities of simulation_thermodynamic_state (L190-233)."""
    raw: np.ndarray
    volume: float

    @property
    def virial(self):
        return self.raw[0:9].reshape(3, 3)

    @property
    def kinetic_momentum(self):
        return self.raw[18:21]

    @property
    def kinetic_energy(self):
        return self.raw[21:24]

    @property
    def potential_energy(self):
        return float(self.raw[24])

    @property
    def mass(self):
        return float(self.raw[25])

    @property
    def particle_count(self):
        return int(self.raw[26])

    @property
    def temperature(self):
        p = self.kinetic_momentum
        return 2.0 * (self.kinetic_energy - 0.5 * p * p / self.mass)

    @property
    def ke_tensor(self):
        ke = self.raw[9:18].reshape(3, 3)
        p = self.kinetic_momentum
        return 2.0 * (ke - 0.5 * np.outer(p, p) / self.mass)

    @property
    def pressure(self):
        return (np.diag(self.ke_tensor) + np.diag(self.virial)) / self.volume

    @property
    def total_energy(self):
        return float(self.kinetic_energy.sum()) + self.potential_energy

    @property
    def temperature_scal(self):
        return float(self.temperature.sum()) / 3.0

    @property
    def full_stress_tensor(self):
        """(virial + kinetic tensor) / volume (thermodynamic_state.h L71-87)."""
        return (self.virial + self.ke_tensor) / self.volume


class Simulation:
    """The grid + domain + species slots shared by the operators, backed by
    one libgbmd context (one GPU, one stream)."""

    def __init__(self, system=None, device: int = 0, species=None):
        self.ctx = _capi.Context(device)
        self.species = species or []
        self.rcut_max = 0.0
        self.ghost_dist_max = 0.0
        self.volume = 0.0
        self.lo = self.hi = np.zeros(3)
        self.mixed = False
        if system is not None:
            self.load(system)

    def load(self, s):
        self.ctx.upload_system(s)
        self.lo, self.hi = np.asarray(s.lo, float), np.asarray(s.hi, float)
        self.volume = float(np.prod(s.hi - s.lo))
        if not self.species:
            self.species = ["T%d" % t for t in range(len(s.masses))]

    def set_precision(self, mixed: bool):
        self.mixed = bool(mixed)
        self.ctx.set_precision(self.mixed)

    def type_index(self, name: str) -> int:
        if name not in self.species:
            raise OperatorError("unknown species %r (species: %s)" % (name, self.species))
        return self.species.index(name)


class Operator:
    name = "operator"
    required = ()

    def __init__(self, **slots):
        for r in self.required:
            if r not in slots:
                raise OperatorError("%s: REQUIRED slot '%s' has no value" % (self.name, r))
        self.slots = slots

    def execute(self, sim: Simulation):
        raise NotImplementedError


class lj_compute_force(Operator):
    name = "lj_compute_force"
    required = ("rcut",)

    def bind(self, sim: Simulation):
        p = self.slots.get("parameters", {})
        eps, sig = quantity(p.get("epsilon", 0.0)), quantity(p.get("sigma", 0.0))
        rcut = quantity(self.slots["rcut"])
        if len(sim.species) > 1 and "type" not in self.slots:
            raise OperatorError("Error: exactly 1 atom type expected (single material) but found %d"
                                % len(sim.species))
        sim.ctx.set_lj(eps, sig, rcut)
        sim.rcut_max = max(sim.rcut_max, rcut)

    def execute(self, sim: Simulation, energy=True, virial=False):
        sim.ctx.compute_forces(energy=energy, virial=virial)


class lj_compute_force_symetric(lj_compute_force):
    """lj_compute_force_symetric (pair_potential_singlemat_symetric.cpp L44,
    slots L335-346): the forces of lj_compute_force, which the reference
    evaluates on a Newton-3 half list, scattering each reaction force under
    per-particle spin locks (`particle_locks`, accepted and unused here).
    The full list gives the same sums up to rounding and is faster on
    GB300, so it is the default (as in the plugin); `half_list: true`
    selects the library's half list, whose reaction forces are added with
    64-bit fixed-point atomics, deterministic as well (mixed precision, one
    lane x 4 entries per load)."""
    name = "lj_compute_force_symetric"

    def bind(self, sim: Simulation):
        super().bind(sim)
        if self.slots.get("half_list", False):
            sim.set_precision(True)
            sim.ctx.set_launch(1, 256, 4)
            sim.ctx.set_newton3(True)


class lj_multi_force(Operator):
    name = "lj_multi_force"
    required = ("rcut",)

    def bind(self, sim: Simulation):
        nt = len(sim.species)
        common = self.slots.get("common_parameters", {"epsilon": 0.0, "sigma": 0.0})
        rcut = quantity(self.slots["rcut"])
        eps = np.full((nt, nt), quantity(common.get("epsilon", 0.0)))
        sig = np.full((nt, nt), quantity(common.get("sigma", 0.0)))
        rc = np.full((nt, nt), rcut)
        if nt * (nt + 1) // 2 > 16:
            raise OperatorError("Too many atom types. Increase MAX_TYPE_PAIR_IDS")
        for item in self.slots.get("parameters", []):
            for k in ("type_a", "type_b", "rcut", "parameters"):
                if k not in item:
                    raise OperatorError("PotentialMultiParameters : missing informations. required information "
                                        "keys are : type_a, type_b, rcut and parameters.")
            a, b = sim.type_index(item["type_a"]), sim.type_index(item["type_b"])
            e, s = quantity(item["parameters"]["epsilon"]), quantity(item["parameters"]["sigma"])
            r = quantity(item["rcut"])
            eps[a, b] = eps[b, a] = e
            sig[a, b] = sig[b, a] = s
            rc[a, b] = rc[b, a] = r
        sim.ctx.set_lj_multi(eps, sig, rc, rcut)
        sim.rcut_max = max(sim.rcut_max, float(rc.max()), rcut)

    def execute(self, sim: Simulation, energy=True, virial=False):
        sim.ctx.compute_forces(energy=energy, virial=virial)


class eam_alloy_force(Operator):
    """eam_rho, eam_rho2emb and eam_force (eam_potential_multimat.cu
    L101-104, L186-232): by default all three in one call (eam_ghost
    single-pass mode: the whole periodic system lives on one GPU, so no halo
    refresh of rho_dEmb is needed between passes).  The split run-file form
    (multi_species_nosym_cs4.msp L8-16: one eam_alloy_force per pass) maps
    onto the library's density pass, which also applies the embedding, and
    its force pass:

      eam_rho (with or without eam_rho2emb)  -> density + embedding pass
      eam_rho2emb alone                      -> nothing (already applied)
      eam_force alone                        -> force pass from the kept F'(rho)
    """
    name = "eam_alloy_force"
    required = ("rcut", "parameters")

    def bind(self, sim: Simulation):
        p = self.slots["parameters"]
        if isinstance(p, Setfl):
            sf = p
        else:
            path = p["file"] if isinstance(p, dict) else p
            sf = read_setfl(path)
        if sf.nelements < len(sim.species):
            raise OperatorError("setfl file has %d elements, %d species declared" % (sf.nelements, len(sim.species)))
        if sf.nelements > 7:
            raise OperatorError("Maximum number of elements is 7")
        rho, emb, frc = (bool(self.slots.get(k, True)) for k in ("eam_rho", "eam_rho2emb", "eam_force"))
        if rho and frc:
            self.passes = "all" if emb else None
        elif rho:
            self.passes = "density"
        elif frc:
            self.passes = "force" if not emb else None
        else:
            self.passes = "none"
        if self.passes is None:
            raise OperatorError("eam_rho2emb %s with eam_rho and eam_force both %s: the embedding runs with "
                                "the density pass" % (emb, rho))
        # eam_symmetry (Newton-3 half list with the rho_j and reaction-force
        # scatter of eam_force_op_multimat.h L162-169, L305-338) selects how
        # the reference evaluates the same sums; here it runs on the full
        # list, which gives the same densities and forces up to rounding and
        # is faster, unless half_list asks for the library's half list (rho_j
        # and reaction forces through fixed-point atomics, deterministic,
        # mixed precision).
        self.symmetry = bool(self.slots.get("eam_symmetry", False))
        rcut = quantity(self.slots["rcut"])
        sim.ctx.set_eam_alloy(sf, rcut, EV * 1.0, EV)
        if self.symmetry and self.slots.get("half_list", False):
            sim.set_precision(True)
            sim.ctx.set_launch(1, 256, 4)
            sim.ctx.set_newton3(True)
        sim.rcut_max = max(sim.rcut_max, rcut)
        if (rho or frc) and self.slots.get("eam_ghost", True):
            sim.ghost_dist_max = max(sim.ghost_dist_max, 2.0 * rcut)

    def execute(self, sim: Simulation, energy=True, virial=False):
        if self.passes != "none":
            sim.ctx.compute_forces(energy=energy, virial=virial, passes=self.passes)


class johnson_force(Operator):
    """The mono-material analytic EAM operator (eam_potential.cu L69-193 with
    johnson.h L28-176): both passes in one call.  `parameters` holds the 19
    EamJohnsonParameters entries as quantities, converted as the reference's
    YAML decoder does (every entry through its unit)."""
    name = "johnson_force"
    required = ("rcut", "parameters")

    def bind(self, sim: Simulation):
        from .systems import JOHNSON_PARAM_NAMES
        p = self.slots["parameters"]
        missing = [k for k in JOHNSON_PARAM_NAMES if k not in p]
        if missing:
            raise OperatorError("johnson_force: missing parameters %s" % ", ".join(missing))
        if len(sim.species) > 1:
            raise OperatorError("johnson_force: single material potential, %d species declared" % len(sim.species))
        rcut = quantity(self.slots["rcut"])
        sim.ctx.set_eam_johnson(np.array([quantity(p[k]) for k in JOHNSON_PARAM_NAMES]), rcut)
        sim.rcut_max = max(sim.rcut_max, rcut)
        sim.ghost_dist_max = max(sim.ghost_dist_max, 2.0 * rcut)

    def execute(self, sim: Simulation, energy=True, virial=False):
        sim.ctx.compute_forces(energy=energy, virial=virial)


class sutton_chen_force(Operator):
    """The mono-material analytic EAM sutton_chen_force (sutton_chen.h
    L30-67 through the two-pass template, eam_potential.cu L69-193): both
    passes in one call.  `parameters` holds c, epsilon, a0, n, m as
    quantities, converted as the reference's YAML decoder does (L73-89)."""
    name = "sutton_chen_force"
    required = ("rcut", "parameters")

    def bind(self, sim: Simulation):
        from .systems import SUTTON_CHEN_PARAM_NAMES
        p = self.slots["parameters"]
        missing = [k for k in SUTTON_CHEN_PARAM_NAMES if k not in p]
        if missing:
            raise OperatorError("sutton_chen_force: missing parameters %s" % ", ".join(missing))
        if len(sim.species) > 1:
            raise OperatorError("sutton_chen_force: single material potential, %d species declared"
                                % len(sim.species))
        rcut = quantity(self.slots["rcut"])
        sim.ctx.set_eam_sutton_chen(np.array([quantity(p[k]) for k in SUTTON_CHEN_PARAM_NAMES]), rcut)
        sim.rcut_max = max(sim.rcut_max, rcut)
        sim.ghost_dist_max = max(sim.ghost_dist_max, 2.0 * rcut)

    def execute(self, sim: Simulation, energy=True, virial=False):
        sim.ctx.compute_forces(energy=energy, virial=virial)


class chunk_neighbors(Operator):
    name = "chunk_neighbors"

    def bind(self, sim: Simulation, rcut_inc: float):
        cs = self.slots.get("config", {}).get("chunk_size", 1)
        if cs != 1:
            raise OperatorError("chunk_size %d: only chunk_size 1 lists are built" % cs)
        sim.ctx.set_skin(quantity(rcut_inc))

    def execute(self, sim: Simulation):
        sim.ctx.build_neighbors()


class check_and_update_particles(Operator):
    """check_and_update_particles (data/config/config_move_particles.msp
    L116-152): trigger_move_particles (particle_displ_over, skin/2) and the
    full update -- wrap, rebin, neighbour list -- when it fires.  Returns the
    trigger's value, as the reference publishes it in trigger_move_particles."""
    name = "check_and_update_particles"

    def execute(self, sim: Simulation) -> bool:
        return sim.ctx.update_neighbors()


class push_f_v_r(Operator):
    name = "push_f_v_r"

    def execute(self, sim: Simulation, dt: float):
        sim.ctx.push_f_v_r(dt, float(self.slots.get("dt_scale", 1.0)))


class push_f_v(Operator):
    name = "push_f_v"

    def execute(self, sim: Simulation, dt: float):
        sim.ctx.push_f_v(dt, float(self.slots.get("dt_scale", 0.5)))


class push_f_v_r_xform_minimization(Operator):
    name = "push_f_v_r_xform_minimization"
    required = ("dt_scale",)

    def execute(self, sim: Simulation, dt: float):
        sim.ctx.push_min(dt, float(self.slots["dt_scale"]), float(self.slots.get("tolF", 0.0)))


class simulation_thermodynamic_state(Operator):
    name = "simulation_thermodynamic_state"

    def execute(self, sim: Simulation) -> ThermodynamicState:
        return ThermodynamicState(sim.ctx.thermo(), sim.volume)


# dump_thermodynamic_state (src/io/dump_thermodynamic_state.cpp L55-120): the
# column set, header and number formats of the reference's
# thermodynamic_state.csv, so runs can be diffed against reference logs.
# Conversion factors from the internal system (angstrom, dalton, picosecond)
# built from CODATA 2018 constants as the reference does (L58-64).
_ATOMIC_MASS = 1.66053906660e-27
_BOLTZMANN = 1.380649e-23
_ELEMENTARY_CHARGE = 1.602176634e-19
THERMO_CONV_TEMPERATURE = 1.0e4 * _ATOMIC_MASS / _BOLTZMANN
THERMO_CONV_ENERGY = 1.0e4 * _ATOMIC_MASS / _ELEMENTARY_CHARGE
THERMO_CONV_PRESSURE = 1.0e4 * _ATOMIC_MASS * 1e30
THERMO_CONV_DENSITY = _ATOMIC_MASS * 1e3 * 1e24
THERMO_HEADER = ("# Step     Time (ps)     Particles  Tot. E. (eV/part)  Kin. E. (eV/part)  Pot. E. (eV/part)  "
                 "Temp. (K) Pxx Pyy Pzz Pxy Pxz Pyz (Pa) A/B/C (ang)    alpha/beta/gamma (deg)     Vol. (ang^3)  "
                 "Rho (g/cm^3)")
_THERMO_FMT = ("%9d % .6e %13d  % .10e  % .10e  % .10e  % 9.12f  % 9.12f  % 9.12f  % 9.12f  % 9.12f  % 9.12f "
               "% 9.12f % 12.12f % 12.12f % 12.12f % 9.12f % 9.12f % 9.12f % 16.12f % 13.12f ")


class dump_thermodynamic_state(Operator):
    """Appends one line per call (the header first when print_header) to
    `thermostate_file`; cubic boxes (identity xform), so the cell angles are
    90 degrees."""
    name = "dump_thermodynamic_state"

    def format_line(self, sim: "Simulation", st: ThermodynamicState, timestep: int, physical_time: float) -> str:
        n = st.particle_count
        P = st.full_stress_tensor * THERMO_CONV_PRESSURE
        lo, hi = np.asarray(sim.lo, float), np.asarray(sim.hi, float)
        A, B, C = (float(v) for v in (hi - lo))
        vol = st.volume
        return _THERMO_FMT % (
            timestep, physical_time, n,
            st.total_energy / n * THERMO_CONV_ENERGY,
            float(st.kinetic_energy.sum()) / n * THERMO_CONV_ENERGY,
            st.potential_energy / n * THERMO_CONV_ENERGY,
            st.temperature_scal / n * THERMO_CONV_TEMPERATURE,
            P[0, 0], P[1, 1], P[2, 2], P[0, 1], P[0, 2], P[1, 2],
            A, B, C, 90.0, 90.0, 90.0, vol, THERMO_CONV_DENSITY * st.mass / vol)

    def execute(self, sim: "Simulation", st: ThermodynamicState, timestep: int, physical_time: float = 0.0):
        path = self.slots.get("thermostate_file", "thermodynamic_state.csv")
        line = self.format_line(sim, st, timestep, physical_time)
        with open(path, "a") as fh:
            if self.slots.get("print_header", True):
                fh.write(THERMO_HEADER + "\n")
            fh.write(line + "\n")
        return line


def verlet_nve(sim: Simulation, nsteps: int, dt: float, rebuild_every: int = 10, thermo_every: int = 0,
               use_graph: bool = False):
    """The verlet_nve graph (config_numerical_schemes.msp L44-52) run on the
    device: first half, rebuild every `rebuild_every` steps, forces with
    force_to_accel, second half; returns the thermo rows (27 doubles each)."""
    return sim.ctx.run_nve(nsteps, dt, rebuild_every, thermo_every, use_graph)


FORCE_OPERATORS = {"lj_compute_force": lj_compute_force, "lj_compute_force_symetric": lj_compute_force_symetric,
                   "lj_multi_force": lj_multi_force,
                   "eam_alloy_force": eam_alloy_force, "johnson_force": johnson_force,
                   "sutton_chen_force": sutton_chen_force}


def compute_force_from_config(cfg: dict) -> Operator:
    """Pick the operator a run file binds to the compute_force slot."""
    slot = cfg.get("compute_force", "nop")
    if slot == "nop":
        raise OperatorError("compute_force is nop: no force operator bound")
    if slot not in FORCE_OPERATORS:
        raise OperatorError("operator '%s' not found" % slot)
    return FORCE_OPERATORS[slot](**cfg.get(slot, {}))

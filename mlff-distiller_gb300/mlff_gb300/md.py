"""Velocity-Verlet NVE molecular dynamics on the GPU.

``VelocityVerletGPU`` advances many independent structures (MD replicas,
or one large periodic box) with the library's float64 integrator
(``mlff_verlet_steps``): per step a half kick, a drift, the neighbour list,
model and force adjoint at the new positions, and a second half kick, with
the per-structure potential and kinetic energy recorded on the device.
Blocks of steps are captured once in a CUDA graph and replayed, so a step
costs no host round trip.

``set_langevin`` (or ``LangevinGPU``) switches the same driver to Langevin
NVT dynamics, the protocol the reference's MD benchmark runs through ASE's
Langevin (benchmarks/md_trajectory.py:407-413): by default ASE's own
propagator (Vanden-Eijnden and Ciccotti, fixed centre of mass;
``mlff_langevin_ase_steps``), or the BAOAB splitting
(``mlff_langevin_steps``); ``set_npt`` (or ``NPTGPU``) to NPT
with the equations of motion of ASE's NPT (Nose-Hoover thermostat,
Parrinello-Rahman barostat; ``mlff_npt_steps``), the reference's NPT
protocol (:415-424), on orthorhombic periodic boxes.

``NVEMDHarness`` mirrors the reference's harness
(testing/nve_harness.py:57-380: Maxwell-Boltzmann start at T, zero
centre-of-mass momentum and angular momentum, VelocityVerlet at dt fs,
energy drift 100 (E_end - E_0) / |E_0|) on top of it.  Energies and the
temperature are recorded every step; positions, velocities and forces
every ``save_interval`` steps.
"""
import ctypes
import time
from typing import Any, Dict, List, Optional

import numpy as np
import torch

from . import _lib, units
from .engine import Batch, _stream_handle


# ------------------------------------------------------------ initial state
def maxwell_boltzmann(masses: np.ndarray, temperature_K: float, rng: np.random.Generator) -> np.ndarray:
    """Velocities (A per internal time unit) with momenta drawn as
    N(0, 1) * sqrt(m kB T) per component (ASE's
    MaxwellBoltzmannDistribution, used at nve_harness.py:158)."""
    m = np.asarray(masses, dtype=np.float64)
    p = rng.standard_normal((m.shape[0], 3)) * np.sqrt(m * units.kB * temperature_K)[:, None]
    return p / m[:, None]


def stationary(vel: np.ndarray, masses: np.ndarray, mol_ptr: np.ndarray) -> np.ndarray:
    """Zero the centre-of-mass momentum of every structure (Stationary,
    nve_harness.py:161-162)."""
    v = vel.copy()
    for b in range(len(mol_ptr) - 1):
        s = slice(mol_ptr[b], mol_ptr[b + 1])
        m = masses[s]
        if m.size:
            v[s] -= (m[:, None] * v[s]).sum(0) / m.sum()
    return v


def zero_rotation(pos: np.ndarray, vel: np.ndarray, masses: np.ndarray, mol_ptr: np.ndarray) -> np.ndarray:
    """Remove the angular momentum about the centre of mass of every
    structure (ZeroRotation, nve_harness.py:164-165): v -= w x (r - r_com)
    with I w = L."""
    v = vel.copy()
    for b in range(len(mol_ptr) - 1):
        s = slice(mol_ptr[b], mol_ptr[b + 1])
        m = masses[s]
        if m.size < 2:
            continue
        r = pos[s] - (m[:, None] * pos[s]).sum(0) / m.sum()
        L = (m[:, None] * np.cross(r, v[s])).sum(0)
        inertia = np.einsum("i,ij,ik->jk", m, r, r)
        inertia = np.trace(inertia) * np.eye(3) - inertia
        omega = np.linalg.lstsq(inertia, L, rcond=None)[0]
        v[s] -= np.cross(omega, r)
    return v


def kinetic_energy(vel: np.ndarray, masses: np.ndarray, mol_ptr: np.ndarray) -> np.ndarray:
    ke = 0.5 * masses[:, None] * vel * vel
    return np.array([ke[mol_ptr[b]:mol_ptr[b + 1]].sum() for b in range(len(mol_ptr) - 1)])


# ------------------------------------------------------------------ driver
class VelocityVerletGPU:
    """Float64 velocity-Verlet for all structures of a batch at once.

    ``model`` is a ``StudentForceField`` on a CUDA device.  ``positions``
    (N, 3) Angstrom, ``numbers`` (N,), ``mol_ptr`` (B + 1) CSR offsets of the
    structures; ``box`` (B, 3) / ``pbc`` (B,) for orthorhombic periodic
    structures; ``masses`` default to the standard atomic weights.
    """

    def __init__(self, model, numbers, positions, mol_ptr, masses=None, box=None, pbc=None,
                 timestep_fs: float = 0.5, capacity_headroom: float = 1.3):
        self.model = model
        self.engine = model.engine()
        self.dev = self.engine.device
        self.lib = self.engine.lib
        self.path = model.path
        z = np.asarray(numbers, dtype=np.int64)
        self.mol_ptr_np = np.asarray(mol_ptr, dtype=np.int64)
        self.N, self.B = int(z.shape[0]), int(self.mol_ptr_np.shape[0] - 1)
        self.masses = units.masses_of(z) if masses is None else np.asarray(masses, dtype=np.float64)
        self.dt = float(timestep_fs) * units.fs
        self.timestep_fs = float(timestep_fs)
        d = self.dev
        self.Z = torch.as_tensor(z, device=d)
        self.mol_ptr = torch.as_tensor(self.mol_ptr_np, device=d)
        self.box = None if box is None else torch.as_tensor(np.asarray(box, np.float32), device=d).reshape(-1, 3)
        self.pbc = None if pbc is None else torch.as_tensor(np.asarray(pbc, np.uint8), device=d).reshape(-1)
        self.pos = torch.as_tensor(np.asarray(positions, np.float64).reshape(self.N, 3), device=d).contiguous()
        self.vel = torch.zeros_like(self.pos)
        self.inv_mass = torch.as_tensor(1.0 / self.masses, device=d)
        self.forces = torch.zeros(self.N, 3, dtype=torch.float32, device=d)
        self.energy = torch.zeros(self.B, dtype=torch.float64, device=d)
        self.kinetic = torch.zeros(self.B, dtype=torch.float64, device=d)
        self.headroom = capacity_headroom
        self.steps_done = 0
        self._graphs: Dict[int, Any] = {}
        self._forces_valid = False
        self.step_counter = torch.zeros(1, dtype=torch.int64, device=d)   # keys the Langevin draws
        self.thermostat: Optional[Dict[str, float]] = None
        self.npt: Optional[Dict[str, float]] = None
        self.box64 = self.zeta = self.eta = self.xi = self.virial = None

    def set_langevin(self, temperature_K: float, friction: float = 0.01, seed: int = 0, scheme: str = "ase",
                     fixcm: bool = True):
        """Langevin NVT from now on: ``friction`` in inverse ASE time units
        (the reference's NVT protocol uses 0.01), target temperature in K;
        ``None`` temperature switches back to NVE.  ``scheme``: "ase" (the
        Vanden-Eijnden-Ciccotti propagator ASE's Langevin integrates, with
        ``fixcm`` as ASE's: centre of mass held in place) or "baoab"."""
        if temperature_K is None:
            self.thermostat = None
            return
        if friction < 0 or temperature_K < 0:
            raise ValueError("friction and temperature must be non-negative")
        if scheme not in ("ase", "baoab"):
            raise ValueError(f"unknown Langevin scheme {scheme!r}: use 'ase' or 'baoab'")
        self.npt = None
        self.thermostat = {"friction": float(friction), "kT": float(units.kB * temperature_K),
                           "seed": int(seed) & 0xFFFFFFFFFFFFFFFF, "scheme": scheme, "fixcm": bool(fixcm)}

    def set_npt(self, temperature_K: Optional[float], externalstress: float = 0.0, ttime: float = 25.0 * units.fs,
                pfactor: float = 75.0 * units.fs ** 2):
        """NPT from now on, with ASE NPT's arguments (the reference's NPT
        protocol: ttime 25 fs, pfactor 75 fs^2, externalstress 0): ttime
        (ASE time units; 0 = no thermostat), pfactor (eV (ASE time)^2 / A^3;
        0 = no barostat), externalstress a scalar pressure in eV/A^3.  Every
        structure must be an orthorhombic periodic box.  ``None``
        temperature switches back to NVE (the box keeps its size)."""
        if temperature_K is None:
            self.npt = None
            return
        if self.box is None or self.pbc is None or not bool(self.pbc.bool().all()):
            raise ValueError("NPT needs every structure periodic (box and pbc)")
        if temperature_K < 0 or ttime < 0 or pfactor < 0 or (ttime > 0 and temperature_K <= 0):
            raise ValueError("NPT needs ttime >= 0, pfactor >= 0 and a positive temperature with a thermostat")
        self.thermostat = None
        self.npt = {"kT": float(units.kB * temperature_K), "ttime": float(ttime), "pfactor": float(pfactor),
                    "pressure": float(externalstress)}
        if self.box64 is None:
            d = self.dev
            self.box64 = self.box.to(torch.float64).clone()
            self.zeta = torch.zeros(self.B, dtype=torch.float64, device=d)
            self.eta = torch.zeros(self.B, 3, dtype=torch.float64, device=d)
            self.xi = torch.zeros(self.B, dtype=torch.float64, device=d)
            self.virial = torch.zeros(self.B, 3, 3, dtype=torch.float64, device=d)
        self._forces_valid = False   # the first NPT step needs the virial

    def volumes(self) -> np.ndarray:
        """Box volumes [B] (A^3)."""
        b = self.box64 if self.box64 is not None else self.box.to(torch.float64)
        return torch.prod(b, dim=1).cpu().numpy()

    def npt_conserved(self) -> np.ndarray:
        """Per structure E + K + P V + 3 n kT (ttime^2 zeta^2 / 2 + xi) +
        pfactor |eta|^2 / 2, the quantity the NPT equations conserve."""
        p = self.npt
        n = np.diff(self.mol_ptr_np).astype(np.float64)
        zeta, xi, eta = self.zeta.cpu().numpy(), self.xi.cpu().numpy(), self.eta.cpu().numpy()
        return (self.energy.cpu().numpy() + self.kinetic.cpu().numpy() + p["pressure"] * self.volumes() +
                3.0 * n * p["kT"] * (0.5 * p["ttime"] ** 2 * zeta ** 2 + xi) +
                0.5 * p["pfactor"] * (eta * eta).sum(axis=1))

    # state
    def set_velocities(self, vel):
        self.vel.copy_(torch.as_tensor(np.asarray(vel, np.float64).reshape(self.N, 3), device=self.dev))

    def initialize_velocities(self, temperature_K: float, seed: int = 0, remove_com_translation: bool = True,
                              remove_com_rotation: bool = True):
        rng = np.random.default_rng(seed)
        v = maxwell_boltzmann(self.masses, temperature_K, rng)
        if remove_com_translation:
            v = stationary(v, self.masses, self.mol_ptr_np)
        if remove_com_rotation:
            v = zero_rotation(self.positions(), v, self.masses, self.mol_ptr_np)
        self.set_velocities(v)

    def snapshot(self) -> Dict[str, torch.Tensor]:
        """Device copies of the integrator state (positions, velocities,
        forces, energies, step count) for restore()."""
        snap = {"pos": self.pos.clone(), "vel": self.vel.clone(), "forces": self.forces.clone(),
                "energy": self.energy.clone(), "kinetic": self.kinetic.clone(), "steps_done": self.steps_done,
                "forces_valid": self._forces_valid, "step_counter": self.step_counter.clone()}
        for k in self._NPT_KEYS:
            if getattr(self, k) is not None:
                snap[k] = getattr(self, k).clone()
        return snap

    _NPT_KEYS = ("box", "box64", "zeta", "eta", "xi", "virial")

    def restore(self, snap: Dict[str, torch.Tensor]):
        """Put a snapshot() back in place (the captured graphs keep working:
        the state tensors are updated in place)."""
        for k in ("pos", "vel", "forces", "energy", "kinetic", "step_counter") + self._NPT_KEYS:
            if k in snap and getattr(self, k) is not None:
                getattr(self, k).copy_(snap[k])
        self.steps_done = snap["steps_done"]
        self._forces_valid = snap["forces_valid"]

    def positions(self) -> np.ndarray:
        return self.pos.cpu().numpy()

    def velocities(self) -> np.ndarray:
        return self.vel.cpu().numpy()

    def get_forces(self) -> np.ndarray:
        return self.forces.cpu().numpy().astype(np.float64)

    def _batch(self) -> Batch:
        return Batch(self.Z, self.pos.to(torch.float32), self.mol_ptr, self.box, self.pbc)

    def compute_forces(self):
        """Energy and forces at the current positions (eager, with the
        edge-capacity check), the start of a trajectory."""
        E, F, V = self.engine.energy_forces(self._batch(), self.path, forces=True, virial=self.npt is not None)
        self.energy.copy_(E)
        self.forces.copy_(F)
        if V is not None:
            self.virial.copy_(V)
        self.kinetic.copy_(torch.as_tensor(kinetic_energy(self.velocities(), self.masses, self.mol_ptr_np),
                                           device=self.dev))
        self._forces_valid = True
        return E.cpu().numpy(), F.cpu().numpy()

    # one library call of n steps on the current stream
    def _call(self, n_steps: int, cap: int, e_trace: Optional[torch.Tensor], k_trace: Optional[torch.Tensor]):
        ws = self.engine.workspace_for(self.N, self.B, cap, self.path)
        st = _lib.MDState()
        st.pos, st.vel = self.pos.data_ptr(), self.vel.data_ptr()
        st.inv_mass, st.forces = self.inv_mass.data_ptr(), self.forces.data_ptr()
        st.energy, st.kinetic = self.energy.data_ptr(), self.kinetic.data_ptr()
        st.energy_trace, st.kinetic_trace = _lib.ptr(e_trace), _lib.ptr(k_trace)
        st.step_counter = self.step_counter.data_ptr()
        sysd = self._batch_sys
        th = self.thermostat
        if self.npt is not None:
            p = self.npt
            ns = _lib.NPTState()
            ns.box, ns.box32 = self.box64.data_ptr(), self.box.data_ptr()
            ns.zeta, ns.eta, ns.xi, ns.virial = (self.zeta.data_ptr(), self.eta.data_ptr(), self.xi.data_ptr(),
                                                 self.virial.data_ptr())
            _lib.check(self.lib.mlff_npt_steps(ctypes.byref(self.engine.dims), self.engine.packed.data_ptr(),
                                               ctypes.byref(sysd), cap, self.path, ctypes.byref(st), ctypes.byref(ns),
                                               ctypes.c_double(self.dt), ctypes.c_double(p["kT"]),
                                               ctypes.c_double(p["ttime"]), ctypes.c_double(p["pfactor"]),
                                               ctypes.c_double(p["pressure"]), n_steps, ws.data_ptr(), ws.numel(),
                                               _stream_handle()))
        elif th is None:
            _lib.check(self.lib.mlff_verlet_steps(ctypes.byref(self.engine.dims), self.engine.packed.data_ptr(),
                                                  ctypes.byref(sysd), cap, self.path, ctypes.byref(st),
                                                  ctypes.c_double(self.dt), n_steps, ws.data_ptr(), ws.numel(),
                                                  _stream_handle()))
        elif th["scheme"] == "ase":
            _lib.check(self.lib.mlff_langevin_ase_steps(ctypes.byref(self.engine.dims), self.engine.packed.data_ptr(),
                                                        ctypes.byref(sysd), cap, self.path, ctypes.byref(st),
                                                        ctypes.c_double(self.dt), ctypes.c_double(th["friction"]),
                                                        ctypes.c_double(th["kT"]), ctypes.c_uint64(th["seed"]),
                                                        1 if th["fixcm"] else 0, n_steps, ws.data_ptr(), ws.numel(),
                                                        _stream_handle()))
        else:
            _lib.check(self.lib.mlff_langevin_steps(ctypes.byref(self.engine.dims), self.engine.packed.data_ptr(),
                                                    ctypes.byref(sysd), cap, self.path, ctypes.byref(st),
                                                    ctypes.c_double(self.dt), ctypes.c_double(th["friction"]),
                                                    ctypes.c_double(th["kT"]), ctypes.c_uint64(th["seed"]), n_steps,
                                                    ws.data_ptr(), ws.numel(), _stream_handle()))

    def _capacity(self) -> int:
        return max(self.engine.capacity(self.N, self.path),
                   int(self.engine.edge_capacity.get(self.path, 0) * self.headroom) + 1024)

    def run(self, n_steps: int, graph: bool = True, block: int = 50, record: bool = True,
            to_host: bool = True) -> Dict[str, np.ndarray]:
        """Advance n_steps.  Returns per-step potential / kinetic energy per
        structure, shape [n_steps, B] (eV), when record is set -- as device
        tensors with to_host=False (e.g. for energy_metrics.replica_energy_stats)."""
        if not self._forces_valid:
            self.compute_forces()
        cap = self._capacity()
        # the library reads the float32 positions of its own buffer; the
        # batch descriptor only carries Z, mol_ptr, box and pbc
        self._pos32 = self.pos.to(torch.float32)
        self._batch_sys = Batch(self.Z, self._pos32, self.mol_ptr, self.box, self.pbc).system()
        self.engine.workspace_for(self.N, self.B, cap, self.path)
        epot = torch.zeros(n_steps, self.B, dtype=torch.float64, device=self.dev) if record else None
        ekin = torch.zeros_like(epot) if record else None
        done = 0
        while done < n_steps:
            k = min(block, n_steps - done)
            et = epot[done:done + k] if record else None
            kt = ekin[done:done + k] if record else None
            if graph and k == block:
                g = self._graph(k, cap, record)
                g["graph"].replay()
                if record:
                    et.copy_(g["e"])
                    kt.copy_(g["k"])
            else:
                self._call(k, cap, et, kt)
            done += k
            # every library call clears the status word first: read it per block
            code, n_edges, where = self.engine.status()
            if code != _lib.OK:
                raise _lib.MLFFError(code, f"device status {code} during MD steps {done - k}..{done} "
                                           f"(edges {n_edges}, index {where}); edge capacity {cap}")
        self.steps_done += n_steps
        if not record:
            return {}
        if not to_host:
            return {"potential_energy": epot, "kinetic_energy": ekin}
        return {"potential_energy": epot.cpu().numpy(), "kinetic_energy": ekin.cpu().numpy()}

    def _graph(self, k: int, cap: int, record: bool):
        ws = self.engine.workspace_for(self.N, self.B, cap, self.path)
        th = self.thermostat
        key = (k, cap, record, ws.data_ptr(), None if th is None else (th["friction"], th["kT"], th["seed"]),
               None if self.npt is None else tuple(sorted(self.npt.items())))
        if key in self._graphs:
            return self._graphs[key]
        # a graph holds the workspace address it was captured with
        self._graphs = {kk: g for kk, g in self._graphs.items() if kk[3] == ws.data_ptr()}
        e = torch.zeros(k, self.B, dtype=torch.float64, device=self.dev) if record else None
        kk = torch.zeros_like(e) if record else None
        g = torch.cuda.CUDAGraph()
        # the state tensors are updated in place by the captured steps
        torch.cuda.synchronize()
        with torch.cuda.graph(g):
            self._call(k, cap, e, kk)
        self._graphs[key] = {"graph": g, "e": e, "k": kk, "ws": ws}
        return self._graphs[key]


class LangevinGPU(VelocityVerletGPU):
    """Langevin NVT driver with ASE Langevin's arguments (timestep in fs,
    temperature_K, friction in inverse ASE time units, fixcm): the
    reference's NVT protocol (benchmarks/md_trajectory.py:407-413) on the
    fused GPU step.  scheme "ase" (default) integrates ASE's propagator,
    "baoab" the BAOAB splitting."""

    def __init__(self, model, numbers, positions, mol_ptr, temperature_K: float, friction: float = 0.01,
                 seed: int = 0, timestep_fs: float = 0.5, fixcm: bool = True, scheme: str = "ase", **kwargs):
        super().__init__(model, numbers, positions, mol_ptr, timestep_fs=timestep_fs, **kwargs)
        self.set_langevin(temperature_K, friction, seed, scheme=scheme, fixcm=fixcm)


class NPTGPU(VelocityVerletGPU):
    """NPT driver with ASE NPT's arguments (timestep in fs, temperature_K,
    externalstress in eV/A^3, ttime, pfactor): the reference's NPT protocol
    (benchmarks/md_trajectory.py:415-424) on the fused GPU step, for
    orthorhombic periodic boxes (box [B,3])."""

    def __init__(self, model, numbers, positions, mol_ptr, box, temperature_K: float, externalstress: float = 0.0,
                 ttime: float = 25.0 * units.fs, pfactor: float = 75.0 * units.fs ** 2, timestep_fs: float = 0.5,
                 **kwargs):
        B = len(np.asarray(mol_ptr)) - 1
        super().__init__(model, numbers, positions, mol_ptr, box=box, pbc=np.ones(B, bool), timestep_fs=timestep_fs,
                         **kwargs)
        self.set_npt(temperature_K, externalstress, ttime, pfactor)


# ----------------------------------------------------------------- harness
class NVEMDHarness:
    """NVE harness with the reference's interface (nve_harness.py:57-380).

    ``atoms`` is an Atoms object (ASE's or the stand-in), ``calculator`` a
    ``StudentForceFieldCalculator``: its model runs the GPU integrator."""

    def __init__(self, atoms, calculator, temperature: float = 300.0, timestep: float = 0.5,
                 trajectory_file=None, log_interval: int = 10, remove_com_motion: bool = True, seed: int = 0):
        self.atoms = atoms.copy()
        self.calculator = calculator
        self.temperature = temperature
        self.timestep_fs = timestep
        self.timestep = timestep * units.fs
        self.trajectory_file = trajectory_file
        self.log_interval = log_interval
        self.remove_com_motion = remove_com_motion
        self.seed = seed
        self.atoms.calc = calculator
        self.reset()

    def reset(self):
        self.trajectory_data: Dict[str, List] = {k: [] for k in (
            "time", "positions", "velocities", "forces", "potential_energy", "kinetic_energy", "total_energy",
            "temperature")}
        self._simulation_complete = False
        self._n_steps = 0
        self._wall_time = 0.0
        self.dynamics: Optional[VelocityVerletGPU] = None

    def _driver(self) -> VelocityVerletGPU:
        a = self.atoms
        pbc = np.asarray(a.get_pbc())
        box = pbc_flag = None
        if pbc.any():
            cell = np.asarray(a.get_cell())
            box, pbc_flag = np.diag(cell)[None, :], np.array([1], np.uint8)
        return VelocityVerletGPU(self.calculator.model, a.get_atomic_numbers(), a.get_positions(),
                                 [0, len(a)], masses=a.get_masses(), box=box, pbc=pbc_flag,
                                 timestep_fs=self.timestep_fs)

    def initialize_velocities(self, temperature=None, remove_com_translation=True, remove_com_rotation=True):
        t = self.temperature if temperature is None else temperature
        rng = np.random.default_rng(self.seed)
        m = self.atoms.get_masses()
        ptr = np.array([0, len(self.atoms)])
        v = maxwell_boltzmann(m, t, rng)
        if remove_com_translation:
            v = stationary(v, m, ptr)
        if remove_com_rotation:
            v = zero_rotation(self.atoms.get_positions(), v, m, ptr)
        self.atoms.set_velocities(v)

    def _record(self, step: int, epot: float, ekin: float, pos=None, vel=None, forces=None):
        n = len(self.atoms)
        self.trajectory_data["time"].append(step * self.timestep_fs / 1000.0)
        self.trajectory_data["potential_energy"].append(epot)
        self.trajectory_data["kinetic_energy"].append(ekin)
        self.trajectory_data["total_energy"].append(epot + ekin)
        self.trajectory_data["temperature"].append(2.0 * ekin / (3 * n * units.kB) if n else 0.0)
        if pos is not None:
            self.trajectory_data["positions"].append(pos)
            self.trajectory_data["velocities"].append(vel)
            self.trajectory_data["forces"].append(forces)

    def run_simulation(self, steps: int, initialize_velocities: bool = True,
                       save_interval: Optional[int] = None) -> Dict[str, Any]:
        if steps <= 0:
            raise ValueError(f"steps must be positive, got {steps}")
        save_interval = save_interval or self.log_interval
        t0 = time.perf_counter()
        try:
            if initialize_velocities:
                self.initialize_velocities()
            drv = self._driver()
            self.dynamics = drv
            drv.set_velocities(self.atoms.get_velocities())
            E, F = drv.compute_forces()
            ek0 = float(kinetic_energy(drv.velocities(), drv.masses, drv.mol_ptr_np)[0])
            self._record(0, float(E[0]), ek0, drv.positions(), drv.velocities(), F.astype(np.float64))
            done = 0
            while done < steps:
                k = min(save_interval, steps - done)
                tr = drv.run(k, graph=True, block=k)
                for i in range(k):
                    last = i == k - 1
                    self._record(done + i + 1, float(tr["potential_energy"][i, 0]), float(tr["kinetic_energy"][i, 0]),
                                 drv.positions() if last else None, drv.velocities() if last else None,
                                 drv.get_forces() if last else None)
                done += k
            self.atoms.set_positions(drv.positions())
            self.atoms.set_velocities(drv.velocities())
            self._simulation_complete = True
            self._n_steps = steps
            self._wall_time = time.perf_counter() - t0
            return self._compute_summary()
        except Exception as e:
            raise RuntimeError(f"NVE MD simulation failed after {len(self.trajectory_data['time'])} steps: {e}") from e

    def _compute_summary(self) -> Dict[str, Any]:
        """nve_harness.py:290-344."""
        td = self.trajectory_data
        if not td["time"]:
            raise RuntimeError("No trajectory data collected")
        times = np.asarray(td["time"])
        et = np.asarray(td["total_energy"])
        temps = np.asarray(td["temperature"])
        e0, ef = et[0], et[-1]
        return {
            "trajectory_data": td, "n_steps": self._n_steps, "total_time_ps": times[-1] - times[0],
            "timestep_fs": self.timestep_fs, "wall_time_s": self._wall_time,
            "energy_drift_pct": 100.0 * (ef - e0) / abs(e0) if e0 != 0 else 0.0,
            "energy_drift_abs": ef - e0, "energy_std": float(np.std(et)), "energy_range": float(np.ptp(et)),
            "avg_temperature": float(np.mean(temps)), "std_temperature": float(np.std(temps)),
            "initial_energy": e0, "final_energy": ef,
            "avg_potential_energy": float(np.mean(td["potential_energy"])),
            "avg_kinetic_energy": float(np.mean(td["kinetic_energy"])),
        }

    @property
    def is_complete(self) -> bool:
        return self._simulation_complete


def replica_drift(potential: np.ndarray, kinetic: np.ndarray, e0_pot: np.ndarray, e0_kin: np.ndarray):
    """Per-structure relative drift 100 (E_end - E_0) / |E_0| and the
    absolute drift, from [steps, B] energy traces and the t = 0 energies."""
    e0 = e0_pot + e0_kin
    e_end = potential[-1] + kinetic[-1]
    return 100.0 * (e_end - e0) / np.abs(e0), e_end - e0

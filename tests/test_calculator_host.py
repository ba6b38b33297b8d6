"""Host-side behaviour of the drop-in ASE calculator and the MD helpers
(no GPU): the reference's error contract (ase_calculator.py:240-244,
405-412, 414-459), the Atoms stand-in's caching, and the initial-velocity
recipe of nve_harness.py:141-170."""
import numpy as np
import pytest
import torch

from mlff_gb300 import md, units
from mlff_gb300.ase_calculator import StudentForceFieldCalculator
from mlff_gb300.ase_compat import Atoms
from mlff_gb300.student_model import StudentForceField


@pytest.fixture()
def ckpt(tmp_path):
    torch.manual_seed(0)
    m = StudentForceField()
    p = tmp_path / "model.pt"
    m.save(p)
    return p


def test_missing_checkpoint():
    with pytest.raises(FileNotFoundError):
        StudentForceFieldCalculator("/nonexistent/model.pt", device="cpu")


def test_jit_without_path(ckpt):
    with pytest.raises(ValueError):
        StudentForceFieldCalculator(ckpt, device="cpu", use_jit=True)


class _Archive(torch.nn.Module):
    """A TorchScript module holding a state_dict under the reference's
    parameter names (what ``torch.jit.save`` of a scripted StudentForceField
    stores)."""

    def __init__(self, sd):
        super().__init__()
        for k, v in sd.items():
            *path, leaf = k.split(".")
            mod = self
            for name in path:
                if not hasattr(mod, name):
                    mod.add_module(name, torch.nn.Module())
                mod = getattr(mod, name)
            mod.register_buffer(leaf, v.clone())

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        return x


def test_jit_archive_loads(tmp_path):
    """use_jit=True with a TorchScript archive (ase_calculator.py:216-237):
    the calculator's model carries the archive's weights, key for key."""
    torch.manual_seed(3)
    sd = StudentForceField().state_dict()
    path = tmp_path / "model_jit.pt"
    torch.jit.save(torch.jit.script(_Archive(sd)), str(path))
    c = StudentForceFieldCalculator(tmp_path / "unused.pt", device="cpu", use_jit=True, jit_path=path)
    got = c.model.state_dict()
    assert set(got) == set(sd)
    for k, v in sd.items():
        assert torch.equal(got[k].cpu(), v), k
    with pytest.raises(FileNotFoundError):
        StudentForceFieldCalculator(tmp_path / "unused.pt", device="cpu", use_jit=True, jit_path=tmp_path / "no.pt")


def test_properties(ckpt):
    c = StudentForceFieldCalculator(ckpt, device="cpu")
    assert c.implemented_properties == ["energy", "forces"]
    c = StudentForceFieldCalculator(ckpt, device="cpu", enable_stress=True)
    assert c.implemented_properties == ["energy", "forces", "stress"]
    assert c.model.num_parameters() == 429596


@pytest.mark.parametrize("bad", ["empty", "z0", "z119", "nan"])
def test_invalid_input_raises_value_error(ckpt, bad):
    c = StudentForceFieldCalculator(ckpt, device="cpu")
    pos = np.zeros((3, 3)) + np.arange(3)[:, None]
    z = np.array([1, 6, 8])
    if bad == "empty":
        pos, z = np.zeros((0, 3)), np.zeros(0, dtype=np.int64)
    elif bad == "z0":
        z = np.array([0, 6, 8])
    elif bad == "z119":
        z = np.array([119, 6, 8])
    else:
        pos[1, 2] = np.nan
    atoms = Atoms(numbers=z, positions=pos)
    atoms.calc = c
    with pytest.raises(ValueError):
        atoms.get_potential_energy()


def test_compute_without_cuda_is_runtime_error(ckpt):
    """Anything but invalid input surfaces as RuntimeError (ase_calculator.py:
    408-412); on a machine without a GPU that is the missing CUDA device --
    there is no CPU fallback."""
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    c = StudentForceFieldCalculator(ckpt, device="cpu")
    atoms = Atoms(numbers=[1, 8, 1], positions=[[0, 0, 0], [0.96, 0, 0], [1.2, 0.9, 0]])
    atoms.calc = c
    with pytest.raises(RuntimeError):
        atoms.get_forces()


def test_atoms_standin_caching():
    from mlff_gb300.ase_compat import Calculator, HAVE_ASE
    if HAVE_ASE:
        pytest.skip("real ASE in use")

    class Counting(Calculator):
        implemented_properties = ["energy", "forces"]

        def __init__(self):
            super().__init__()
            self.calls = 0

        def calculate(self, atoms=None, properties=("energy",), system_changes=()):
            Calculator.calculate(self, atoms, properties, system_changes)
            self.calls += 1
            self.results = {"energy": float(atoms.positions.sum()), "forces": -atoms.positions.copy()}

    a = Atoms(numbers=[1, 1], positions=[[0, 0, 0], [0.7, 0, 0]])
    a.calc = Counting()
    e1 = a.get_potential_energy()
    a.get_forces()
    assert a.calc.calls == 1
    a.set_positions(a.get_positions() + 0.1)
    assert a.get_potential_energy() != e1
    assert a.calc.calls == 2


def test_units():
    # 1 fs in Angstrom * sqrt(amu / eV) units
    assert abs(units.fs - 0.09822694788464063) < 1e-9
    assert units.ATOMIC_MASSES[1] == 1.008 and units.ATOMIC_MASSES[8] == 15.999


def test_initial_velocities():
    rng = np.random.default_rng(0)
    n, B = 64, 32
    ptr = np.arange(B + 1) * n
    pos = rng.normal(size=(n * B, 3)) * 3.0
    m = units.masses_of(rng.choice([1, 6, 7, 8], size=n * B))
    v = md.maxwell_boltzmann(m, 300.0, rng)
    # equipartition: <m v^2> = 3 kB T per atom, within sampling error
    t = (m[:, None] * v * v).sum() / (3 * len(m) * units.kB)
    assert abs(t - 300.0) < 15.0
    v = md.stationary(v, m, ptr)
    v = md.zero_rotation(pos, v, m, ptr)
    for b in range(B):
        s = slice(ptr[b], ptr[b + 1])
        p = (m[s, None] * v[s]).sum(0)
        r = pos[s] - (m[s, None] * pos[s]).sum(0) / m[s].sum()
        L = (m[s, None] * np.cross(r, v[s])).sum(0)
        assert np.abs(p).max() < 1e-10
        assert np.abs(L).max() < 1e-8


def test_oracle_verlet_harmonic():
    """The restated integrator on a harmonic oscillator: second order in dt,
    energy bounded."""
    from oracle.md import velocity_verlet
    k, m0 = 2.0, 3.0

    def f(r):
        return np.array([0.5 * k * (r * r).sum()]), -k * r

    r0, v0 = np.array([[1.0, 0, 0]]), np.array([[0.0, 0.5, 0]])
    w = np.sqrt(k / m0)
    errs = []
    for dt in (0.02, 0.01):
        n = int(round(2.0 / dt))
        r, v, F, ep, ek = velocity_verlet(r0, v0, [m0], f, dt, n, np.array([0, 1]))
        t = n * dt
        exact = np.array([np.cos(w * t), 0.5 / w * np.sin(w * t), 0])
        errs.append(np.abs(r[0] - exact).max())
        e = ep[:, 0] + ek[:, 0]
        assert np.ptp(e) < 1e-3
    assert 3.5 < errs[0] / errs[1] < 4.5


def test_oracle_philox_known_answers():
    """Philox4x32-10 against the known-answer vectors published with the
    generator's reference implementation (counter, key -> output)."""
    from oracle.philox import philox4x32_10
    kat = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
           ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
           ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
            (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, out in kat:
        got = philox4x32_10(np.array(ctr, np.uint32), np.array(key, np.uint32))
        assert tuple(int(x) for x in got) == out


def test_oracle_langevin_normals_and_equipartition():
    """The Box-Muller normals are standard normal, and BAOAB of free
    particles relaxes the kinetic energy to 3/2 kT per atom."""
    from oracle.md import langevin_baoab
    from oracle.philox import langevin_normals
    xi = np.concatenate([langevin_normals(7, s, 2000) for s in range(5)])
    assert abs(xi.mean()) < 0.02 and abs(xi.std() - 1.0) < 0.02
    n, kT = 500, units.kB * 300.0
    m = np.full(n, 12.0)

    def free(r):
        return np.zeros(1), np.zeros_like(r)

    r, v, F, ep, ek = langevin_baoab(np.zeros((n, 3)), np.zeros((n, 3)), m, free, 1.0 * units.fs, 0.05 / units.fs,
                                     kT, 3, 0, 400, np.array([0, n]))
    T_kin = ek[200:, 0].mean() / (1.5 * n * kT)
    assert abs(T_kin - 1.0) < 0.05


def test_student_calculator_contract(tmp_path):
    """Generic StudentCalculator: constructor errors as the reference's, and a
    foreign dict-in/dict-out module evaluated as the reference does."""
    from mlff_gb300.student_calculator import StudentCalculator
    with pytest.raises(ValueError):
        StudentCalculator(device="cpu")
    with pytest.raises(FileNotFoundError):
        StudentCalculator(model_path=tmp_path / "missing.pth", device="cpu")
    with pytest.raises(ValueError):
        StudentCalculator(model=lambda: 3, device="cpu")

    class Toy(torch.nn.Module):   # energy = sum |r|^2, forces = -2 r
        def forward(self, inp):
            r = inp["positions"]
            return {"energy": (r * r).sum().reshape(1), "forces": -2.0 * r}

    calc = StudentCalculator(model=Toy(), device="cpu")
    a = Atoms(numbers=[1, 8], positions=[[0.0, 0, 0], [1.0, 2.0, 0]])
    a.calc = calc
    assert abs(a.get_potential_energy() - 5.0) < 1e-6
    np.testing.assert_allclose(a.get_forces(), [[0, 0, 0], [-2.0, -4.0, 0]], atol=1e-6)
    assert calc.n_calls >= 1
    # a state_dict that is not a StudentForceField needs model_class
    torch.save({"model_state_dict": Toy().state_dict()}, tmp_path / "toy.pth")
    with pytest.raises(RuntimeError):
        StudentCalculator(model_path=tmp_path / "toy.pth", device="cpu")


def _soft_pairs(n_side=3, a=2.0, seed=0):
    """Periodic soft Gaussian pair potential (E = sum exp(-d^2/2)), its
    forces and strain derivative, for the NPT oracle checks."""
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(n_side)] * 3, indexing="ij"), -1).reshape(-1, 3) * a
    pos = g + 0.3 * rng.normal(size=g.shape)

    def ff(r, L):
        d = r[:, None, :] - r[None, :, :]
        d -= L * np.round(d / L)
        e = np.exp(-0.5 * (d * d).sum(-1))
        np.fill_diagonal(e, 0.0)
        return 0.5 * e.sum(), (e[:, :, None] * d).sum(1), -0.5 * np.einsum("ij,ija,ijb->ab", e, d, d)

    return pos, ff


def test_oracle_npt_conserves_extended_energy():
    """The NPT restatement (thermostat and barostat on) conserves E + K +
    P V + 3 n kT (ttime^2 zeta^2 / 2 + xi) + pfactor |eta|^2 / 2 to the
    accuracy of its splitting, while the box changes."""
    from oracle.md import npt_conserved, npt_melchionna
    pos, ff = _soft_pairs()
    n = pos.shape[0]
    L0 = np.full(3, 6.0)
    m = np.ones(n)
    v = 0.3 * np.random.default_rng(1).normal(size=pos.shape)
    kT, tt, pf, P = 0.05, 0.5, 200.0, 0.01
    E, F, W = ff(pos, L0)
    H0 = npt_conserved(E, 0.5 * (v * v).sum(), 216.0, n, kT, tt, pf, P, 0.0, np.zeros(3), 0.0)
    o = npt_melchionna(pos, v, m, L0, ff, 0.01, kT, tt, pf, P, 300)
    H1 = npt_conserved(o["epot"][-1], o["ekin"][-1], o["volume"][-1], n, kT, tt, pf, P, o["zeta"], o["eta"],
                       o["xi"])
    assert abs(o["volume"][-1] - 216.0) > 1.0
    assert abs(H1 - H0) < 1e-3, (H0, H1)


def test_oracle_npt_strain_derivative_is_the_energy_change_under_strain():
    """The force field's W (used by the barostat) is dE/d(strain):
    E((1 + e) r, (1 + e) L) against central differences."""
    pos, ff = _soft_pairs(seed=2)
    L = np.full(3, 6.0)
    _, _, W = ff(pos, L)
    for a in range(3):
        h = 1e-6
        S = np.zeros((3, 3))
        S[a, a] = h
        ep = ff(pos @ (np.eye(3) + S).T, L * (1 + np.diag(S)))[0]
        em = ff(pos @ (np.eye(3) - S).T, L * (1 - np.diag(S)))[0]
        assert abs((ep - em) / (2 * h) - W[a, a]) < 1e-6

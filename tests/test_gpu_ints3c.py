"""The engine's integral kernels (gdfjk_three_index_device, gdfjk_metric_device) against the
host integral provider, which the oracle tests pin to the reference's golden energies.

Both evaluate the same McMurchie–Davidson expressions in FP64 (different loop orders and
fused multiply-adds), so they agree to a few units in the last place of the largest
integral: the bar is 1e-13 of max|(P|mn)|.  Covered: pure and Cartesian bases, f primary
and g fitting shells (cc-pVTZ / cc-pVTZ-JKFIT), contracted s shells of 8 primitives, the
Schwarz shell mask, row ranges that cut through shells, and a column map."""
import numpy as np
import pytest

from psi4_gb300.basis import BasisSet
from psi4_gb300.device_init import DeviceBasis, metric_device, three_index_device
from psi4_gb300.ints import Integrals
from tests.helpers import reference_values, system

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
DEV = torch.device("cuda:0")
REL = 1e-13


def _three_index(pb, ab, ref_shape, **kw):
    out = torch.zeros(ref_shape, dtype=torch.float64, device=DEV)
    pd, ad = DeviceBasis(pb), DeviceBasis(ab)
    three_index_device(ad, pd, out.data_ptr(), ref_shape[1], **kw)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("name,basis", [("h2o", "cc-pvtz"), ("h2o_2", "cc-pvdz"), ("h2o_8", "cc-pvdz")])
def test_three_index_matches_host(ints_built, jk_built, name, basis):
    mol, pb, ab, ints, df = system(name, basis)
    sm = df.sparsity.shell_mask
    ref = ints.three_index(shell_mask=sm)
    got = _three_index(pb, ab, ref.shape, shell_mask=sm)
    d = np.abs(got - ref).max()
    print(f"{name}/{basis}: naux {ab.nbf}, {ref.shape[1]} pairs, max|(P|mn)| {np.abs(ref).max():.3f}, max|d| {d:.2e}")
    assert d <= REL * max(1.0, np.abs(ref).max())


def test_three_index_all_pairs_cartesian(ints_built, jk_built):
    """Cartesian components (no solid-harmonic transform), every shell pair."""
    mol, _, _, _, _ = system("h2o", "cc-pvtz")
    pb = BasisSet.build(mol, "cc-pvtz", puream=False)
    ab = BasisSet.fitting_for(mol, pb)
    ints = Integrals(mol, pb, ab)
    ref = ints.three_index()
    got = _three_index(pb, ab, ref.shape)
    assert np.abs(got - ref).max() <= REL * max(1.0, np.abs(ref).max())


def test_three_index_row_range_and_column_map(ints_built, jk_built):
    """Rows p0..p1 cutting through shells, and the significant pairs' columns through a map
    (the screened build's layout)."""
    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz")
    sp = df.sparsity
    p0, p1 = 7, 61
    ref = ints.three_index(shell_mask=sp.shell_mask, p0=p0, p1=p1)
    r, c = np.tril_indices(pb.nbf)
    sig = np.flatnonzero(sp.pair_mask[r, c])
    rng = np.random.default_rng(0)
    sig = np.sort(rng.choice(sig, size=sig.size // 2, replace=False))
    col_map = np.full(r.size, -1, dtype=np.int64)
    col_map[sig] = np.arange(sig.size)
    col_d = torch.from_numpy(col_map).to(DEV)
    out = torch.zeros((p1 - p0, sig.size), dtype=torch.float64, device=DEV)
    three_index_device(DeviceBasis(ab), DeviceBasis(pb), out.data_ptr(), sig.size, shell_mask=sp.shell_mask, p0=p0,
                       p1=p1, col_map_ptr=col_d.data_ptr())
    got = out.cpu().numpy()
    assert np.abs(got - ref[:, sig]).max() <= REL * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("basis", ["cc-pvtz", "cc-pvdz"])
def test_metric_matches_host(ints_built, jk_built, basis):
    mol, pb, ab, ints, df = system("h2o", basis)
    ref = ints.metric()
    n = ab.nbf
    out = torch.zeros((n, n), dtype=torch.float64, device=DEV)
    metric_device(DeviceBasis(ab), out.data_ptr(), n)
    got = out.cpu().numpy()
    d = np.abs(got - ref).max()
    print(f"metric {basis}-jkfit: naux {n}, max|M| {np.abs(ref).max():.3f}, max|d| {d:.2e}")
    assert d <= REL * np.abs(ref).max()
    part = torch.zeros((20, n), dtype=torch.float64, device=DEV)
    metric_device(DeviceBasis(ab), part.data_ptr(), n, p0=5, p1=25)
    assert np.abs(part.cpu().numpy() - ref[5:25]).max() <= REL * np.abs(ref).max()


def test_device_integrals_scf2_energy(ints_built, jk_built):
    """scf2 (water cc-pVTZ) with B built entirely on the device: integrals, metric, tensor-core
    metric contraction; the reference energy within its tolerance."""
    from psi4_gb300.device_init import build_device_B
    from psi4_gb300.jk import GpuDFJK
    from psi4_gb300.scf import core_hamiltonian, rhf

    ref = reference_values()["scf2"]
    mol, pb, ab, ints, df = system("h2o_scf2", "cc-pvtz")
    dd = build_device_B(mol, pb, ab, ints=ints, keep_rows=ab.nbf)
    assert "three_index_device_s" in dd.timings
    assert np.abs(dd.rows - df.B_tri).max() < 2e-12
    jk = GpuDFJK.from_engine(dd.engine)
    r = rhf(jk, core_hamiltonian(ints), ints.overlap(), mol.nelectron // 2, mol.nuclear_repulsion_energy(),
            e_conv=1e-10, d_conv=1e-8)
    print(f"scf2 from device integrals: {r.energy:.12f} ref {ref['energy']:.12f}")
    assert abs(r.energy - ref["energy"]) < ref["tolerance"]


@pytest.mark.parametrize("name,basis", [("h2o", "cc-pvtz"), ("h2o_8", "cc-pvdz")])
def test_metric_power_device_matches_host(ints_built, jk_built, name, basis):
    """J^-1/2 with Matrix::power's truncation on the device eigensolver against the host
    restatement.  Both eigensolvers are backward stable (exact for M + dM, |dM| ~ eps |M|), and
    the metric is ill-conditioned, so the two J^-1/2 differ by ~1e-10 of their largest entry
    (7.9e-9 of 55 on water cc-pVTZ); what B depends on, J^-1/2 M J^-1/2 = 1, holds equally
    well for both."""
    from psi4_gb300.device_init import metric_power_device
    from psi4_gb300.dfhelper import DEFAULT_CONDITION, metric_power

    mol, pb, ab, ints, df = system(name, basis)
    M = ints.metric()
    ref = metric_power(M, -0.5, DEFAULT_CONDITION)
    got = metric_power_device(torch.from_numpy(M).to(DEV), -0.5, DEFAULT_CONDITION).cpu().numpy()
    d = np.abs(got - ref).max()
    I = np.eye(M.shape[0])
    e_ref, e_got = np.abs(ref @ M @ ref - I).max(), np.abs(got @ M @ got - I).max()
    print(f"{name}/{basis}: max|J^-1/2| {np.abs(ref).max():.2f}, max|d| {d:.2e}, |J^-1/2 M J^-1/2 - 1| host {e_ref:.1e} "
          f"device {e_got:.1e}")
    assert d < 1e-9 * np.abs(ref).max()
    assert e_got < 10 * max(e_ref, 1e-12)


def test_device_metric_power_scf2_energy(ints_built, jk_built):
    """scf2 with J^-1/2 from the device eigensolver: the reference energy within its tolerance."""
    from psi4_gb300.device_init import build_device_B
    from psi4_gb300.jk import GpuDFJK
    from psi4_gb300.scf import core_hamiltonian, rhf

    ref = reference_values()["scf2"]
    mol, pb, ab, ints, df = system("h2o_scf2", "cc-pvtz")
    dd = build_device_B(mol, pb, ab, ints=ints, metric_power_on="device")
    assert "metric_power_device_s" in dd.timings
    jk = GpuDFJK.from_engine(dd.engine)
    r = rhf(jk, core_hamiltonian(ints), ints.overlap(), mol.nelectron // 2, mol.nuclear_repulsion_energy(),
            e_conv=1e-10, d_conv=1e-8)
    print(f"scf2 with the device J^-1/2: {r.energy:.12f} ref {ref['energy']:.12f}")
    assert abs(r.energy - ref["energy"]) < ref["tolerance"]


@pytest.mark.parametrize("name,basis", [("h2o_2", "cc-pvdz"), ("h2o", "cc-pvtz")])
def test_three_index_grad_matches_host(ints_built, jk_built, name, basis):
    """sum G3[P][mn] d(P|mn)/dx on the device (derivative kernels, atomics) against the host
    provider for a seeded random density over the significant shell pairs."""
    from psi4_gb300.device_init import three_index_grad_device

    mol, pb, ab, ints, df = system(name, basis)
    sm = df.sparsity.shell_mask
    rng = np.random.default_rng(7)
    G3 = rng.standard_normal((ab.nbf, pb.nbf * (pb.nbf + 1) // 2))
    ref = ints.three_index_grad(G3, shell_mask=sm)
    g = torch.zeros((mol.natom, 3), dtype=torch.float64, device=DEV)
    Gd = torch.from_numpy(G3).to(DEV)
    three_index_grad_device(DeviceBasis(ab), DeviceBasis(pb), Gd.data_ptr(), G3.shape[1], mol.natom, g.data_ptr(),
                            shell_mask=sm)
    got = g.cpu().numpy()
    d = np.abs(got - ref).max()
    print(f"{name}/{basis}: max|grad| {np.abs(ref).max():.3e} max|d| {d:.2e}")
    assert d <= 1e-12 * max(1.0, np.abs(ref).max())
    assert np.abs(got.sum(0)).max() <= 1e-10 * max(1.0, np.abs(ref).max())  # translational invariance


@pytest.mark.parametrize("basis", ["cc-pvtz", "cc-pvdz"])
def test_metric_grad_matches_host(ints_built, jk_built, basis):
    from psi4_gb300.device_init import metric_grad_device

    mol, pb, ab, ints, df = system("h2o_2", basis)
    rng = np.random.default_rng(3)
    G2 = rng.standard_normal((ab.nbf, ab.nbf))
    G2 = G2 + G2.T
    ref = ints.metric_grad(G2)
    g = torch.zeros((mol.natom, 3), dtype=torch.float64, device=DEV)
    Gd = torch.from_numpy(G2).to(DEV)
    metric_grad_device(DeviceBasis(ab), Gd.data_ptr(), ab.nbf, mol.natom, g.data_ptr())
    got = g.cpu().numpy()
    d = np.abs(got - ref).max()
    print(f"metric grad {basis}: max|grad| {np.abs(ref).max():.3e} max|d| {d:.2e}")
    assert d <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("name,basis", [("h2o_2", "cc-pvdz"), ("h2o", "cc-pvtz")])
def test_potential_grad_matches_host(ints_built, jk_built, name, basis):
    """The nuclear-attraction derivatives with point charges on the device against the host
    provider, for a seeded random symmetric density."""
    from psi4_gb300.device_init import potential_grad_device

    mol, pb, ab, ints, df = system(name, basis)
    rng = np.random.default_rng(5)
    D = rng.standard_normal((pb.nbf, pb.nbf))
    D = D + D.T
    ref = ints.potential_grad(D)
    r, c = np.tril_indices(pb.nbf)
    Dp = np.where(r == c, 1.0, 2.0) * D[r, c]
    g = torch.zeros((mol.natom, 3), dtype=torch.float64, device=DEV)
    Dd = torch.from_numpy(np.ascontiguousarray(Dp)).to(DEV)
    potential_grad_device(DeviceBasis(pb), Dd.data_ptr(), mol, g.data_ptr())
    got = g.cpu().numpy()
    d = np.abs(got - ref).max()
    print(f"{name}/{basis} potential grad: max|g| {np.abs(ref).max():.3e} max|d| {d:.2e}")
    assert d <= 1e-12 * max(1.0, np.abs(ref).max())

"""The reference's stored DF-SCF energies reached through the GPU engine (native FP64 and
the emulated-FP64 form) instead of the oracle JK."""
import pytest

from psi4_gb300.jk import GpuDFJK
from tests.helpers import reference_values
from tests.test_golden import _rhf_energy_zm

pytestmark = pytest.mark.gpu


def _gpu(precision):
    def make(df):
        jk = GpuDFJK.from_tensor(df)
        jk.set_precision(precision)
        jk.initialize()
        return jk
    return make


@pytest.mark.parametrize("precision", ["fp64", "fp64-emulated"])
@pytest.mark.parametrize("basis", ["cc-pvdz", "cc-pvtz"])
def test_gpu_dfmp2_2_h2(ints_built, jk_built, precision, basis):
    ref = reference_values()["dfmp2_2_h2"]
    r, _ = _rhf_energy_zm(ref["zmatrix"], basis, _gpu(precision))
    print(f"H2 {basis} {precision}: {r.energy:.14f} ref {ref['energy'][basis]:.14f}")
    assert abs(r.energy - ref["energy"][basis]) < ref["tolerance"]


@pytest.mark.parametrize("precision", ["fp64", "fp64-emulated"])
def test_gpu_scf2_and_dfomp2_1_water(ints_built, jk_built, precision):
    vals = reference_values()
    r, _ = _rhf_energy_zm(vals["scf2"]["zmatrix"], vals["scf2"]["basis"], _gpu(precision))
    assert abs(r.energy - vals["scf2"]["energy"]) < vals["scf2"]["tolerance"]
    ref = vals["dfomp2_1_water"]
    r, _ = _rhf_energy_zm(ref["zmatrix"], ref["basis"], _gpu(precision))
    assert abs(r.energy - ref["energy"]) < 1e-9


@pytest.mark.parametrize("subtype", ["INCORE", "OUT_OF_CORE"])
@pytest.mark.parametrize("screening", ["SCHWARZ", "DENSITY", "CSAM", "NONE"])
def test_gpu_comprehensive_jk_screening(ints_built, jk_built, subtype, screening):
    """The MEM_DF rows of tests/pytests/test_comprehensive_jk_screening.py: singlet O2
    cc-pVTZ, df_scf_guess off, one DF energy for every screening and subtype (6 decimals);
    SCREENING=DENSITY raises psi4's error.  OUT_OF_CORE runs with B in Grace memory."""
    from psi4_gb300.jk import build_jk
    from psi4_gb300.scf import core_hamiltonian, rhf
    from tests.helpers import system

    ref = reference_values()["scf5_singlet_df"]
    mol, pb, ab, ints, _ = system("o2", "cc-pvtz")
    opts = {"SCF_SUBTYPE": subtype, "SCREENING": screening, "DF_SCF_GUESS": False}
    if screening == "DENSITY":
        with pytest.raises(RuntimeError, match="SCREENING=DENSITY has not been implemented for MEM_DF."):
            build_jk(pb, ab, mol, opts)
        return
    jk = build_jk(pb, ab, mol, opts)
    jk.initialize()
    assert jk.b_host == (subtype == "OUT_OF_CORE")
    r = rhf(jk, core_hamiltonian(ints), ints.overlap(), mol.nelectron // 2, mol.nuclear_repulsion_energy(),
            e_conv=1e-10, d_conv=1e-8)
    print(f"O2 {subtype}+{screening}: {r.energy:.12f} ref {ref['energy']:.12f}")
    assert abs(r.energy - ref["energy"]) < ref["tolerance"]

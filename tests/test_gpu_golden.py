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

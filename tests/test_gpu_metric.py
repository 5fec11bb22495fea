"""The metric contraction B = J^-1/2 (P|mn) on the tensor cores (gdfjk_metric_contract_device):
the emulated-FP64 digit products run as a general product, against FP64 references.

Tolerances: the eight 7-bit digits are fixed point relative to each row of the metric and
each column of (P|mn) (per run of 1024 aux functions), so the digit error scales with
max|row| max|col| (about 2^-52 of it per term) rather than with each term; the double-float
epilogue adds ~2^-45 of |B|.  On real integrals, where J^-1/2 entries reach ~50 and cancel
to |B| ~ 1, B agrees with the FP64 product to 2e-12 (a CPU model of this arithmetic gives
4e-14 for water cc-pVTZ; seven digits would give 7e-11) and the SCF energy matches the
reference's value."""
import numpy as np
import pytest

from psi4_gb300.jk import DFJKEngine, GdfjkError, GpuDFJK
from tests.helpers import reference_values, system

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
DEV = torch.device("cuda:0")


def _raw_three_index(ints, df):
    """(P|mn) in the packed-triangle order, screened pairs zero (as the DF tensor is built)."""
    A = ints.three_index(shell_mask=df.sparsity.shell_mask)
    r, c = np.tril_indices(df.nbf)
    A[:, ~df.sparsity.pair_mask[r, c]] = 0.0
    return A


def _contract(eng, Jm, A, ld=None, out=None, accumulate=False):
    Jd = torch.from_numpy(np.ascontiguousarray(Jm)).to(DEV)
    Ad = torch.from_numpy(np.ascontiguousarray(A)).to(DEV)
    ncols = A.shape[1]
    if out is None:
        out = torch.empty((Jm.shape[0], ld or ncols), dtype=torch.float64, device=DEV)
    eng.metric_contract(Jd.data_ptr(), Ad.data_ptr(), ncols, out.data_ptr(), ldp=ncols, ldb=out.shape[1],
                        accumulate=accumulate)
    return out


@pytest.mark.parametrize("name,basis", [("h2o_8", "cc-pvdz"), ("h2o_scf2", "cc-pvtz")])
def test_metric_contract_real_integrals(ints_built, jk_built, name, basis):
    """B from the raw integrals and J^-1/2 agrees with the FP64 product of the DF tensor."""
    mol, pb, ab, ints, df = system(name, basis)
    A = _raw_three_index(ints, df)
    eng = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    B = _contract(eng, df.Jmhalf, A).cpu().numpy()
    err = np.abs(B - df.B_tri).max()
    print(f"{name}/{basis}: naux {df.naux}, {A.shape[1]} pairs, max|B| {np.abs(df.B_tri).max():.3f}, max|dB| {err:.2e}")
    assert err < 2e-12


def test_metric_contract_scf2_energy(ints_built, jk_built):
    """scf2 (water cc-pVTZ) with B built by the tensor-core metric contraction: the reference
    energy within its tolerance, through the native FP64 J/K."""
    from psi4_gb300.scf import core_hamiltonian, rhf

    ref = reference_values()["scf2"]
    mol, pb, ab, ints, df = system("h2o_scf2", "cc-pvtz")
    eng = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    B = _contract(eng, df.Jmhalf, _raw_three_index(ints, df))
    eng.upload_device(B.data_ptr())
    jk = GpuDFJK.from_engine(eng)
    r = rhf(jk, core_hamiltonian(ints), ints.overlap(), mol.nelectron // 2, mol.nuclear_repulsion_energy(),
            e_conv=1e-10, d_conv=1e-8)
    print(f"scf2 with the device metric contraction: {r.energy:.12f} ref {ref['energy']:.12f}")
    assert abs(r.energy - ref["energy"]) < ref["tolerance"]


@pytest.mark.parametrize("naux,ncols", [(37, 1), (37, 200), (300, 1000), (2500, 777)])
def test_metric_contract_random(jk_built, naux, ncols):
    """Random operands with magnitudes spread over six decades, sizes off every tile multiple,
    naux 2500 over three accumulation runs; reference: the FP64 library product."""
    g = torch.Generator(device=DEV)
    g.manual_seed(naux + ncols)
    Jm = torch.randn((naux, naux), dtype=torch.float64, device=DEV, generator=g)
    Jm *= torch.pow(10.0, torch.rand((naux, 1), dtype=torch.float64, device=DEV, generator=g) * 6 - 3)
    A = torch.randn((naux, ncols), dtype=torch.float64, device=DEV, generator=g)
    A *= torch.pow(10.0, torch.rand((1, ncols), dtype=torch.float64, device=DEV, generator=g) * 6 - 3)
    ref = Jm @ A
    bound = (Jm.abs().amax(dim=1, keepdim=True) * A.abs().amax(dim=0, keepdim=True)) * naux ** 0.5
    eng = DFJKEngine(8, naux, None)
    B = torch.empty_like(ref)
    eng.metric_contract(Jm.data_ptr(), A.data_ptr(), ncols, B.data_ptr())
    rel = ((B - ref).abs() / bound).max().item()
    print(f"naux {naux} ncols {ncols}: max |dB| / (max|row| max|col| sqrt(naux)) = {rel:.2e}")
    assert rel < 1e-13


def test_metric_contract_accumulate_ld_chunks(jk_built, monkeypatch):
    """Leading dimensions wider than the column count leave the extra columns alone;
    accumulate adds to B; column chunks (a tiny digit budget) give bitwise the same B."""
    naux, ncols, ld = 130, 450, 512
    g = torch.Generator(device=DEV)
    g.manual_seed(5)
    Jm = torch.randn((naux, naux), dtype=torch.float64, device=DEV, generator=g)
    A = torch.randn((naux, ncols), dtype=torch.float64, device=DEV, generator=g)
    eng = DFJKEngine(8, naux, None)
    B0 = torch.randn((naux, ld), dtype=torch.float64, device=DEV, generator=g)
    B = B0.clone()
    eng.metric_contract(Jm.data_ptr(), A.data_ptr(), ncols, B.data_ptr(), ldb=ld, accumulate=True)
    assert torch.equal(B[:, ncols:], B0[:, ncols:])
    err = (B[:, :ncols] - (B0[:, :ncols] + Jm @ A)).abs().max().item()
    assert err < 1e-11  # |B| ~ 11 here
    B1 = torch.empty((naux, ncols), dtype=torch.float64, device=DEV)
    eng.metric_contract(Jm.data_ptr(), A.data_ptr(), ncols, B1.data_ptr())
    monkeypatch.setenv("GDFJK_OZ_GEMM_CHUNK_GB", "0.0001")  # 128 columns a chunk
    B2 = torch.empty_like(B1)
    eng.metric_contract(Jm.data_ptr(), A.data_ptr(), ncols, B2.data_ptr())
    assert torch.equal(B1, B2)


def test_metric_contract_rejects_bad_leading_dimension(jk_built):
    eng = DFJKEngine(8, 16, None)
    x = torch.zeros((16, 64), dtype=torch.float64, device=DEV)
    with pytest.raises(GdfjkError, match="leading dimension"):
        eng.metric_contract(x.data_ptr(), x.data_ptr(), 64, x.data_ptr(), ldp=32)


@pytest.mark.parametrize("transb", [False, True])
def test_general_product_both_operand_orders(jk_built, transb):
    """gdfjk_gemm_device: C (+)= A op(B) for op(B) = B and B^T, sizes off every tile multiple,
    an inner dimension over several accumulation runs, magnitudes spread over six decades;
    an inner dimension taken in two accumulated chunks gives the same C (the way the gradient
    forms Gamma A^T)."""
    M, N, K = 300, 277, 3100
    g = torch.Generator(device=DEV)
    g.manual_seed(17 + int(transb))
    A = torch.randn((M, K), dtype=torch.float64, device=DEV, generator=g)
    A *= torch.pow(10.0, torch.rand((M, 1), dtype=torch.float64, device=DEV, generator=g) * 6 - 3)
    Bm = torch.randn((N, K) if transb else (K, N), dtype=torch.float64, device=DEV, generator=g)
    opB = Bm.T if transb else Bm
    ref = A @ opB
    bound = (A.abs().amax(dim=1, keepdim=True) * opB.abs().amax(dim=0, keepdim=True)) * K ** 0.5
    eng = DFJKEngine(8, 8, None)
    C = torch.empty((M, N), dtype=torch.float64, device=DEV)
    ldb = K if transb else N
    eng.gemm(A.data_ptr(), K, Bm.data_ptr(), ldb, C.data_ptr(), N, M, N, K, transb=transb)
    rel = ((C - ref).abs() / bound).max().item()
    print(f"transb {transb}: max |dC| / (max|row| max|col| sqrt(K)) = {rel:.2e}")
    assert rel < 1e-13
    if transb:  # the inner dimension in two chunks, accumulated
        C2 = torch.empty_like(C)
        k1 = 1024
        eng.gemm(A.data_ptr(), K, Bm.data_ptr(), K, C2.data_ptr(), N, M, N, k1, transb=True)
        eng.gemm(A[:, k1:].data_ptr(), K, Bm[:, k1:].data_ptr(), K, C2.data_ptr(), N, M, N, K - k1, transb=True,
                 accumulate=True)
        assert ((C2 - ref).abs() / bound).max().item() < 1e-13
    eng.close()

"""Failure paths of the engine, driven from the host (no GPU fault, trap or hang).

psi4 reports these conditions as PSIEXCEPTIONs (dfhelper.cc:167-173 for memory; the
MemDF -> DiskDF fallback of jk.cc:211-226 when B does not fit); the engine returns status
codes and keeps the handle usable:

* non-finite input  -> GDFJK_ERR_NUMERIC (native FP64: the finite check of J/K; the
  tensor-core forms: their exponent kernels, which would otherwise turn NaN into finite
  digit garbage)
* the host watchdog -> GDFJK_ERR_TIMEOUT while the work is still running, then OK
* refused device allocations (gdfjk_debug_refuse_allocations) -> the release-and-retry path
  (the tensor-core forms give the other form's copy of B back, the native FP64 K both), and
  GDFJK_ERR_OOM when the retry is refused too; the refusal placed at every allocation of a
  build in turn
* a bounded device wait that runs out (gdfjk_debug_wait_probe) -> GDFJK_ERR_DEVICE
"""
import numpy as np
import pytest

from psi4_gb300 import _jkabi as abi
from psi4_gb300 import _native
from psi4_gb300.jk import DFJKEngine, GdfjkError
from tests.helpers import system

pytestmark = pytest.mark.gpu

FORMS = {"native": abi.DO_J | abi.DO_K, "emulated": abi.DO_J | abi.DO_K | abi.EMULATED,
         "mixed": abi.DO_J | abi.DO_K | abi.MIXED}


def _orbitals(nbf, nocc, seed):
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((nbf, nocc)))
    return np.ascontiguousarray(q * 0.5)


def _engine(df):
    eng = DFJKEngine(df.nbf, df.naux, None)
    eng.upload_qtri(df.B_tri)
    return eng


@pytest.fixture(autouse=True)
def _no_refusals_left():
    yield
    _native.jk_lib().gdfjk_debug_refuse_allocations(0, 0)


@pytest.mark.parametrize("form", sorted(FORMS))
def test_nan_in_C_is_numeric_error_and_handle_stays_usable(ints_built, jk_built, form):
    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz", 1e-12)
    eng = _engine(df)
    C = _orbitals(df.nbf, 10, 1)
    J0, K0, _ = eng.compute(C, mode=FORMS[form])
    bad = C.copy()
    bad[3, 4] = np.nan
    with pytest.raises(GdfjkError) as ei:
        eng.compute(bad, mode=FORMS[form])
    assert ei.value.code == abi.GDFJK_ERR_NUMERIC
    J1, K1, _ = eng.compute(C, mode=FORMS[form])
    assert np.array_equal(J0, J1) and np.array_equal(K0, K1)
    eng.close()


def test_watchdog_times_out_then_the_build_completes(jk_built):
    torch = pytest.importorskip("torch")
    nbf, naux, nocc = 384, 1856, 80  # (H2O)_16 cc-pVDZ shape: a native FP64 build of ~0.1 s
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    B = torch.empty((naux, nbf * (nbf + 1) // 2), dtype=torch.float64, device="cuda").normal_(0, 0.02, generator=gen)
    C = torch.randn((nbf, nocc), dtype=torch.float64, device="cuda", generator=gen) * 0.1
    eng = DFJKEngine(nbf, naux, None)
    eng.upload_device(B.data_ptr())
    J = torch.empty((nbf, nbf), dtype=torch.float64, device="cuda")
    K = torch.empty_like(J)
    mode = abi.DO_J | abi.DO_K
    eng.compute_device(C.data_ptr(), None, nocc, nocc, mode, None, J.data_ptr(), K.data_ptr())
    eng.synchronize()
    Jr, Kr = J.clone(), K.clone()
    J.zero_()
    K.zero_()
    eng.compute_device(C.data_ptr(), None, nocc, nocc, mode, None, J.data_ptr(), K.data_ptr())
    with pytest.raises(GdfjkError) as ei:
        eng.synchronize(timeout_s=1e-4)
    assert ei.value.code == abi.GDFJK_ERR_TIMEOUT
    eng.synchronize(timeout_s=600.0)  # the work itself finishes
    assert torch.equal(J, Jr) and torch.equal(K, Kr)
    eng.close()


def _refuse(count, after=0):
    """Set the injection; returns how many refusals of the previous setting were unused."""
    pending = _native.jk_lib().gdfjk_debug_refuse_allocations(after, count)
    assert pending >= 0
    return pending


def test_oom_releases_the_other_form_and_retries(ints_built, jk_built):
    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz", 1e-12)
    C = _orbitals(df.nbf, 10, 2)
    ref = _engine(df)
    _, Ke, _ = ref.compute(C, mode=FORMS["emulated"])
    _, Km, _ = ref.compute(C, mode=FORMS["mixed"])
    ref.close()
    # the emulated form's first allocation is refused: the mixed form's copy of B is released
    # and the build is retried once, with the same result as without the refusal
    eng = _engine(df)
    eng.compute(C, mode=FORMS["mixed"])
    _refuse(1)
    _, K1, _ = eng.compute(C, mode=FORMS["emulated"])
    assert np.array_equal(K1, Ke)
    # the retry refused too: GDFJK_ERR_OOM, and the handle still builds afterwards
    eng.close()
    eng = _engine(df)
    eng.compute(C, mode=FORMS["mixed"])
    _refuse(2)
    with pytest.raises(GdfjkError) as ei:
        eng.compute(C, mode=FORMS["emulated"])
    assert ei.value.code == abi.GDFJK_ERR_OOM
    _refuse(0)
    _, K2, _ = eng.compute(C, mode=FORMS["emulated"])
    assert np.array_equal(K2, Ke)
    # and the other direction: the mixed form's allocation refused after an emulated build
    eng.close()
    eng = _engine(df)
    eng.compute(C, mode=FORMS["emulated"])
    _refuse(1)
    _, K3, _ = eng.compute(C, mode=FORMS["mixed"])
    assert np.array_equal(K3, Km)
    eng.close()


@pytest.mark.parametrize("form", ["emulated", "mixed", "native"])
@pytest.mark.parametrize("count", [1, 2])
def test_refusal_at_every_allocation_of_a_build(ints_built, jk_built, form, count):
    """`count` allocations refused after the first `after` of a build, for every `after` up to
    the number the build makes: the call either succeeds (the retry absorbed a single
    refusal) or returns GDFJK_ERR_OOM, and the next build on the same handle gives exactly
    the undisturbed result (no buffer is left missing behind a capacity that claims it)."""
    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz", 1e-12)
    C = _orbitals(df.nbf, 10, 3)
    ref = _engine(df)
    Jr, Kr, _ = ref.compute(C, mode=FORMS[form])
    ref.close()
    other = "mixed" if form == "emulated" else "emulated"
    outcomes = []
    for after in range(0, 60):
        eng = _engine(df)
        eng.compute(C, mode=FORMS[other])  # a copy of B the retry path can release
        _refuse(count, after)
        try:
            eng.compute(C, mode=FORMS[form])
            outcomes.append("ok")
        except GdfjkError as ex:
            assert ex.code == abi.GDFJK_ERR_OOM, str(ex)
            outcomes.append("oom")
        unused = _refuse(0)
        J, K, _ = eng.compute(C, mode=FORMS[form])
        assert np.array_equal(J, Jr) and np.array_equal(K, Kr), (after, outcomes)
        eng.close()
        if unused == count:
            break  # the build made no more than `after` allocations: every point was covered
    else:
        pytest.fail("the sweep did not reach the end of the build's allocations")
    assert outcomes[-1] == "ok" and len(outcomes) >= 2  # at least one refusal point inside the build
    if count == 2:
        assert "oom" in outcomes  # the retry is refused too


def test_bounded_wait_runs_out_and_the_kernel_returns(ints_built, jk_built):
    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz", 1e-12)
    eng = _engine(df)
    C = _orbitals(df.nbf, 10, 4)
    J0, K0, _ = eng.compute(C, mode=FORMS["emulated"])
    L = _native.jk_lib()
    rc = L.gdfjk_debug_wait_probe(eng.h, 0.05)
    assert rc == abi.GDFJK_ERR_DEVICE
    assert b"flag 2" in L.gdfjk_last_error(eng.h)
    J1, K1, _ = eng.compute(C, mode=FORMS["emulated"])
    assert np.array_equal(J0, J1) and np.array_equal(K0, K1)
    eng.close()


def test_released_split_copy_keeps_the_incremental_history(ints_built, jk_built):
    """Memory pressure (gdfjk_trim, or the other form's OOM retry) drops the precision form's
    split copy of B but not the K it increments: the next increment after a release gives
    bitwise the increment without one."""
    from psi4_gb300.jk import density_difference_factor

    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz", 1e-12)
    C1 = _orbitals(df.nbf, 10, 5)
    C2 = _orbitals(df.nbf, 10, 6)
    U, npos = density_difference_factor(C2, C1)
    out = []
    for release in (False, True):
        eng = _engine(df)
        eng.compute_incremental(C1, C1, C1.shape[1], reset=True)
        if release:
            eng.trim()
        out.append(eng.compute_incremental(C2, U, npos, reset=False))
        eng.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])

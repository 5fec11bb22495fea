"""The precision form's build schedule (`scf.PrecisionSchedule`) driving the RHF loop, on the
CPU.  A JK stand-in computes every build exactly with the oracle and records the form and the
incremental flag that the schedule set before it, so the schedule's host logic is checked
without a GPU:

* split-BF16 increments from the guess, one FP64 anchor (kept as the increments' base) once
  the orbital gradient falls below anchor_d, increments again, then FP64 full rebuilds;
* nothing but FP64 rebuilds after the first of them, and convergence accepted only on an FP64
  build that follows another one (the final two Fock builds are FP64);
* the JK settings of every build match the mode the log reports, and the converged energy is
  the plain FP64 SCF's."""
import numpy as np

from oracle import dfjk_ref
from psi4_gb300.scf import PrecisionSchedule, core_hamiltonian, rhf
from tests.helpers import system

SETTINGS = {"mixed": ("mixed", True), "anchor": ("fp64-emulated", True), "fp64": ("fp64-emulated", False)}


class RecordingJK(dfjk_ref.OracleJK):
    def __init__(self, *args):
        super().__init__(*args)
        self.precision, self.incremental, self.builds = "fp64", False, []

    def set_precision(self, p):
        self.precision = p

    def set_incremental(self, v):
        self.incremental = bool(v)

    def compute(self):
        self.builds.append((self.precision, self.incremental))
        super().compute()


def _run(schedule):
    mol, pb, ab, ints, df = system("h2o")
    H, S = core_hamiltonian(ints), ints.overlap()
    nocc, e_nuc = mol.nelectron // 2, mol.nuclear_repulsion_energy()
    plain = rhf(dfjk_ref.OracleJK(df.to_pQq(), df.sparsity, df.nbf, df.naux), H, S, nocc, e_nuc)
    jk = RecordingJK(df.to_pQq(), df.sparsity, df.nbf, df.naux)
    res = rhf(jk, H, S, nocc, e_nuc, schedule=schedule)
    return plain, res, jk


def test_schedule_order_and_final_fp64_builds(ints_built):
    sched = PrecisionSchedule(fp64_precision="fp64-emulated")
    plain, res, jk = _run(sched)
    assert res.converged and plain.converged
    assert abs(res.energy - plain.energy) < 1e-9
    modes = [e["precision"] for e in res.log]
    assert len(modes) == res.iterations == len(jk.builds)
    assert [SETTINGS[m] for m in modes] == jk.builds
    # increments first, one anchor, then FP64 rebuilds only
    assert modes[0] == "mixed"
    assert modes.count("anchor") == sched.n_anchor == 1  # water cc-pVDZ: m m m m m A m m m m F F
    first_fp64 = modes.index("fp64")
    assert all(m != "fp64" for m in modes[:first_fp64])
    assert all(m == "fp64" for m in modes[first_fp64:])
    assert len(modes) - first_fp64 >= 2
    assert sched.n_mixed == modes.count("mixed")
    assert sched.n_fp64 == modes.count("fp64") + modes.count("anchor")
    # the anchor comes after the orbital gradient fell below anchor_d, not before
    ia = modes.index("anchor")
    assert res.log[ia - 1]["dnorm"] < sched.anchor_d
    assert all(res.log[i]["dnorm"] >= sched.anchor_d for i in range(ia - 1))


def test_schedule_without_anchor_and_with_a_mixed_cap(ints_built):
    """anchor_d None: no anchor; max_mixed caps the increments before the FP64 switch."""
    sched = PrecisionSchedule(anchor_d=None, max_mixed=3, fp64_precision="fp64-emulated")
    plain, res, jk = _run(sched)
    assert res.converged
    assert abs(res.energy - plain.energy) < 1e-9
    modes = [e["precision"] for e in res.log]
    assert modes[:3] == ["mixed"] * 3 and "anchor" not in modes
    assert all(m == "fp64" for m in modes[3:]) and len(modes) >= 5
    assert [SETTINGS[m] for m in modes] == jk.builds

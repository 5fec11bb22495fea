"""Shared builders for the tests: small molecules with real integrals."""
import functools
import json
import os

import numpy as np

from psi4_gb300.basis import BasisSet
from psi4_gb300.dfhelper import build_df_tensor, prepare_sparsity, DFTensor, metric_power
from psi4_gb300.ints import Integrals
from psi4_gb300.molecule import water_c2v, water_cluster, zmatrix

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def reference_values():
    with open(os.path.join(GOLDEN, "reference_values.json")) as fh:
        return json.load(fh)


@functools.lru_cache(maxsize=None)
def system(name: str, basis: str = "cc-pvdz", cutoff: float = 1e-12):
    """(mol, primary, aux, ints, df) for a named small system."""
    if name == "h2o":
        mol = zmatrix(["O", "H 1 1.0", "H 1 1.0 2 103.1"])
    elif name == "h2o_scf2":
        mol = zmatrix(["O", "H 1 1.0", "H 1 1.0 2 104.5"])
    elif name == "h2o_c2v":
        mol = water_c2v(1.0, 104.5)
    elif name == "o2":
        mol = zmatrix(["O", "O 1 1.1"])
    elif name == "h2o_2":
        mol = water_cluster(2, 1, 1, seed=3)
    elif name == "h2o_2_far":
        mol = water_cluster(2, 1, 1, seed=3, spacing=9.0)
    elif name == "h2o_8":
        mol = water_cluster(2, 2, 2, seed=0)
    else:
        raise KeyError(name)
    pb = BasisSet.build(mol, basis)
    ab = BasisSet.fitting_for(mol, pb)
    ints = Integrals(mol, pb, ab)
    df = build_df_tensor(mol, pb, ab, cutoff=cutoff, ints=ints)
    return mol, pb, ab, ints, df


def random_orbitals(nbf, nocc, seed=0):
    rng = np.random.default_rng(seed)
    return rng.random((nbf, nocc))

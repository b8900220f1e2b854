"""Results JSON (dmrg_results_json.mojo, dmrg_json_loader.mojo) and the oracle's bond
entropies (no GPU).

The writer's text is compared with the layout of dmrg_results_json.mojo:36-86
written out here for one input; the loader reads it back (with and without the
optional keys).  The oracle's entropies are pinned on a product state (0) and a
GHZ state (ln 2 at every bond).
"""
import math

import numpy as np
import pytest

from chemtensor_mojo_gb300 import results as R
from oracle import observables as ob

EXPECTED = """{
  "impl": "gb300",
  "model": "heisenberg_xxz",
  "params": {
    "nsites": 4,
    "d": 2,
    "J": 1.0,
    "D": 0.5,
    "h": 0.0,
    "num_sweeps": 3,
    "maxiter_lanczos": 20,
    "chi_max": 16,
    "tol_split": 1e-10
  },
  "energy_final": -1.5,
  "en_sweeps": [-1.25, -1.5, -1.5],
  "entropy": [0.5, 0.6931471805599453, 0.5],
  "bond_dims": [1, 2, 4, 2, 1],
  "norm": 1.0
}
"""


def params(tol=1e-10):
    return R.DMRGJsonParams(nsites=4, d=2, J=1.0, D=0.5, h=0.0, num_sweeps=3, maxiter_lanczos=20, chi_max=16,
                            tol_split=tol)


def test_writer_layout_and_round_trip(tmp_path):
    text = R.dmrg_results_to_json_string("gb300", "heisenberg_xxz", params(), -1.5, [-1.25, -1.5, -1.5],
                                         [0.5, math.log(2.0), 0.5], [1, 2, 4, 2, 1], 1.0)
    assert text == EXPECTED
    path = tmp_path / "res.json"
    R.save_dmrg_results_to_json(str(path), "gb300", "heisenberg_xxz", params(), -1.5, [-1.25, -1.5, -1.5],
                                [0.5, math.log(2.0), 0.5], [1, 2, 4, 2, 1], 1.0)
    ref = R.load_dmrg_reference(str(path))
    assert (ref.impl, ref.model, ref.nsites, ref.d, ref.chi_max, ref.num_sweeps, ref.maxiter_lanczos) == \
        ("gb300", "heisenberg_xxz", 4, 2, 16, 3, 20)
    assert (ref.J, ref.D, ref.h, ref.tol_split, ref.energy_final, ref.norm) == (1.0, 0.5, 0.0, 1e-10, -1.5, 1.0)
    assert ref.en_sweeps == [-1.25, -1.5, -1.5]
    assert ref.bond_dims == [1, 2, 4, 2, 1]
    assert ref.entropy == [0.5, math.log(2.0), 0.5]
    R.print_dmrg_reference_info(ref)


def test_optional_keys_omitted(tmp_path):
    text = R.dmrg_results_to_json_string("gb300", "ising", params(tol=-1.0), -1.0, [-1.0], [], [1, 1], 1.0)
    assert '"tol_split"' not in text and '"entropy"' not in text
    path = tmp_path / "res.json"
    path.write_text(text)
    ref = R.load_dmrg_reference(str(path))
    assert ref.tol_split == -1.0 and ref.entropy == []


def test_entropy_known_answers():
    L, d = 5, 2
    prod = np.zeros(d ** L)
    prod[3] = 1.0
    assert ob.bond_entropies_statevector(prod, L, d) == pytest.approx([0.0] * (L - 1), abs=1e-14)
    ghz = np.zeros(d ** L)
    ghz[0] = ghz[-1] = 1.0 / math.sqrt(2.0)
    assert ob.bond_entropies_statevector(ghz, L, d) == pytest.approx([math.log(2.0)] * (L - 1), rel=1e-14)
    assert R.entropy_from_schmidt([1.0, 1.0]) == pytest.approx(math.log(2.0), rel=1e-15)
    assert R.entropy_from_schmidt([0.0, 0.0]) == 0.0

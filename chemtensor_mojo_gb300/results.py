"""DMRG results in the reference's JSON schema, and bond entropies on the device.

* ``DMRGJsonParams`` / ``dmrg_results_to_json_string`` / ``save_dmrg_results_to_json``
  src/algorithms/dmrg_results_json.mojo:11-102 (same keys, key order and layout,
  so C, Mojo and these files compare with a diff or a tolerance script)
* ``DMRGReference`` / ``load_dmrg_reference`` / ``print_dmrg_reference_info``
  src/tests/algorithms/dmrg/dmrg_json_loader.mojo:13-127
* ``mps_bond_entropies``: the schema's optional ``entropy`` list, which the
  reference reserves but never fills (src/main.mojo:662).  Von Neumann entropy
  -sum p ln p, p = s^2 / sum s^2, of the Schmidt values s at each inner bond,
  from a device right-normalisation followed by a left-to-right SVD sweep.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from typing import List, Sequence

from .dense_tensor import DenseTensor, DeviceContext, create_dense_tensor, dense_tensor_dot, dense_tensor_svd_trunc, \
    get_context
from .mps_state import MatrixProductState, mps_right_normalize


@dataclass
class DMRGJsonParams:
    """The 'params' object (dmrg_results_json.mojo:11-23); tol_split < 0 omits the key."""
    nsites: int
    d: int
    J: float
    D: float
    h: float
    num_sweeps: int
    maxiter_lanczos: int
    chi_max: int
    tol_split: float = -1.0


def _fmt_float(x: float) -> str:
    return repr(float(x))


def dmrg_results_to_json_string(impl: str, model: str, params: DMRGJsonParams, energy_final: float,
                                en_sweeps: Sequence[float], entropy: Sequence[float], bond_dims: Sequence[int],
                                norm: float) -> str:
    """The JSON text, line for line in the layout of dmrg_results_json.mojo:36-86."""
    out = "{\n"
    out += f'  "impl": "{impl}",\n'
    out += f'  "model": "{model}",\n'
    out += '  "params": {\n'
    out += f'    "nsites": {int(params.nsites)},\n'
    out += f'    "d": {int(params.d)},\n'
    out += f'    "J": {_fmt_float(params.J)},\n'
    out += f'    "D": {_fmt_float(params.D)},\n'
    out += f'    "h": {_fmt_float(params.h)},\n'
    out += f'    "num_sweeps": {int(params.num_sweeps)},\n'
    out += f'    "maxiter_lanczos": {int(params.maxiter_lanczos)},\n'
    out += f'    "chi_max": {int(params.chi_max)}'
    if params.tol_split >= 0.0:
        out += f',\n    "tol_split": {_fmt_float(params.tol_split)}'
    out += "\n  },\n"
    out += f'  "energy_final": {_fmt_float(energy_final)},\n'
    out += '  "en_sweeps": [' + ", ".join(_fmt_float(e) for e in en_sweeps) + "],\n"
    if len(entropy) > 0:
        out += '  "entropy": [' + ", ".join(_fmt_float(e) for e in entropy) + "],\n"
    out += '  "bond_dims": [' + ", ".join(str(int(b)) for b in bond_dims) + "],\n"
    out += f'  "norm": {_fmt_float(norm)}\n'
    out += "}\n"
    return out


def save_dmrg_results_to_json(path: str, impl: str, model: str, params: DMRGJsonParams, energy_final: float,
                              en_sweeps: Sequence[float], entropy: Sequence[float], bond_dims: Sequence[int],
                              norm: float) -> None:
    """dmrg_results_json.mojo:89-102."""
    with open(path, "w") as f:
        f.write(dmrg_results_to_json_string(impl, model, params, energy_final, en_sweeps, entropy, bond_dims,
                                            norm))


@dataclass
class DMRGReference:
    """Loaded results (dmrg_json_loader.mojo:13-36); tol_split is -1 when absent, entropy empty."""
    impl: str
    model: str
    nsites: int
    d: int
    J: float
    D: float
    h: float
    num_sweeps: int
    maxiter_lanczos: int
    chi_max: int
    tol_split: float
    energy_final: float
    en_sweeps: List[float] = field(default_factory=list)
    bond_dims: List[int] = field(default_factory=list)
    norm: float = 0.0
    entropy: List[float] = field(default_factory=list)


def load_dmrg_reference(filepath: str) -> DMRGReference:
    """dmrg_json_loader.mojo:51-104."""
    with open(filepath) as f:
        data = json.load(f)
    p = data["params"]
    return DMRGReference(
        impl=str(data["impl"]), model=str(data["model"]), nsites=int(p["nsites"]), d=int(p["d"]),
        J=float(p["J"]), D=float(p["D"]), h=float(p["h"]), num_sweeps=int(p["num_sweeps"]),
        maxiter_lanczos=int(p["maxiter_lanczos"]), chi_max=int(p["chi_max"]),
        tol_split=float(p["tol_split"]) if "tol_split" in p else -1.0,
        energy_final=float(data["energy_final"]), en_sweeps=[float(x) for x in data["en_sweeps"]],
        bond_dims=[int(x) for x in data["bond_dims"]], norm=float(data["norm"]),
        entropy=[float(x) for x in data.get("entropy", [])])


def print_dmrg_reference_info(ref: DMRGReference) -> None:
    """dmrg_json_loader.mojo:107-127."""
    print("DMRG Reference:")
    print("  impl:", ref.impl)
    print("  model:", ref.model)
    print("  nsites:", ref.nsites)
    print("  d:", ref.d)
    print(f"  params: J={ref.J} D={ref.D} h={ref.h}")
    print("  num_sweeps:", ref.num_sweeps)
    print("  chi_max:", ref.chi_max)
    print("  energy_final:", ref.energy_final)
    print("  norm:", ref.norm)
    print("  bond_dims: [" + ", ".join(str(b) for b in ref.bond_dims) + "]")


def entropy_from_schmidt(s: Sequence[float]) -> float:
    w = [float(x) * float(x) for x in s]
    tot = sum(w)
    if tot <= 0.0:
        return 0.0
    return -sum((p / tot) * math.log(p / tot) for p in w if p > 0.0)


def mps_bond_entropies(mps: MatrixProductState, ctx: DeviceContext | None = None) -> List[float]:
    """Entropies of the L-1 inner bonds (from mps_schmidt_values)."""
    return [entropy_from_schmidt(s.tolist()) for s in mps_schmidt_values(mps, ctx)]


def mps_schmidt_values(mps: MatrixProductState, ctx: DeviceContext | None = None) -> List["np.ndarray"]:
    """Schmidt values of the L-1 inner bonds of the normalised state, descending, as NumPy
    arrays.  Right-normalise, then sweep left to right: M_i = C_{i-1} A_i = U S V^T
    (FP64 device Jacobi SVD, no truncation), S are the Schmidt values of bond i+1 and
    C_i = S V^T goes on to the next site.  (Not U^T M_i: a one-sided Jacobi's columns
    U = X / sigma for sigma below eps |M|_F are rounding noise, not orthonormal, and
    U^T M_i would feed that noise into every later bond.)"""
    ctx = ctx or get_context()
    psi = mps_right_normalize(ctx, mps)
    N = psi.num_sites()
    d = psi.physical_dim
    out: List = []
    carry: DenseTensor | None = None
    for i in range(N - 1):
        A = psi.sites[i].tensor
        Dl, _, Dr = A.shape
        if carry is None:
            M = A.reshape([Dl * d, Dr])
        else:
            k = carry.shape[0]
            M = create_dense_tensor(ctx, [k, d * Dr])
            dense_tensor_dot(M, carry, A.reshape([Dl, d * Dr]), ctx)
            M = M.reshape([k * d, Dr])
        U, S, Vt, c = dense_tensor_svd_trunc(M, ctx, chi_max=1 << 30, eps_trunc=0.0)
        out.append(S.to_numpy().reshape(-1).copy())
        carry = DenseTensor(Vt.storage.view(c, Dr).mul(S.storage.view(c, 1)).reshape(-1), [c, Dr])
    return out

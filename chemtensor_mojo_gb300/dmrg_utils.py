"""Gauge-invariant DMRG checks (src/algorithms/dmrg_utils.mojo:18-91) on the device.

* ``energy``        <psi|H|psi> / <psi|psi>
* ``variance_op``   <H^2> - <H>^2 through mpo_compose
* ``fidelity``      |<psi1|psi2>|
* ``observe_sz``    <Sz(i)> = <Z(i)> / 2
* ``observe_sz_sz`` <Sz(i) Sz(j)> = <Z(i) Z(j)> / 4
* ``observe_sx_sx`` <Sx(i) Sx(j)> = <X(i) X(j)> / 4
"""
from __future__ import annotations

from .dense_tensor import DeviceContext, get_context
from .environments import expectation_value_normalized, mps_overlap, variance
from .mps_state import (MatrixProductOperator, MatrixProductState, create_single_site_op_mpo,
                        create_two_site_op_mpo)

PAULI_Z = (1.0, 0.0, 0.0, -1.0)
PAULI_X = (0.0, 1.0, 1.0, 0.0)


def energy(mps: MatrixProductState, mpo: MatrixProductOperator, ctx: DeviceContext | None = None) -> float:
    return expectation_value_normalized(mps, mpo, ctx)


def variance_op(mps: MatrixProductState, mpo: MatrixProductOperator, ctx: DeviceContext | None = None) -> float:
    return variance(mps, mpo, ctx)


def fidelity(mps1: MatrixProductState, mps2: MatrixProductState, ctx: DeviceContext | None = None) -> float:
    return abs(mps_overlap(mps1, mps2, ctx))


def observe_sz(mps: MatrixProductState, site_i: int, ctx: DeviceContext | None = None) -> float:
    ctx = ctx or get_context()
    op = create_single_site_op_mpo(ctx, mps.num_sites(), site_i, PAULI_Z)
    return 0.5 * expectation_value_normalized(mps, op, ctx)


def observe_sz_sz(mps: MatrixProductState, site_i: int, site_j: int, ctx: DeviceContext | None = None) -> float:
    ctx = ctx or get_context()
    op = create_two_site_op_mpo(ctx, mps.num_sites(), site_i, site_j, PAULI_Z, PAULI_Z)
    return 0.25 * expectation_value_normalized(mps, op, ctx)


def observe_sx_sx(mps: MatrixProductState, site_i: int, site_j: int, ctx: DeviceContext | None = None) -> float:
    ctx = ctx or get_context()
    op = create_two_site_op_mpo(ctx, mps.num_sites(), site_i, site_j, PAULI_X, PAULI_X)
    return 0.25 * expectation_value_normalized(mps, op, ctx)

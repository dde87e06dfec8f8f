"""The 64-bit index instantiations of every kernel, which states over 2^31 amplitudes
take (src/types.hpp's Index is 64-bit), checked against the oracle on small states:
dfs_set_wide_index(1) makes every state take them, and the statevector, density-matrix,
reduction, adjoint-gradient, paired-gadget and allocation-free parity tests run again under it."""
import pytest

import test_adjoint_gpu as adj
import test_dm_gpu as dm
import test_fusion_gpu as fusion
import test_sv_gpu as sv
import test_zz_no_alloc as noalloc

PRECISIONS = sv.PRECISIONS

pytestmark = pytest.mark.gpu


@pytest.fixture
def wide(dfs):
    dfs.set_wide_index(True)
    try:
        yield
    finally:
        dfs.set_wide_index(False)


SV_TESTS = [sv.test_one_targ_all_positions, sv.test_many_ctrl_one_targ, sv.test_swap, sv.test_pauli_tensor,
            sv.test_pauli_gadget, sv.test_pauli_z_only_and_identity, sv.test_phase_gadget,
            sv.test_many_targ_whole_register]
DM_TESTS = [dm.test_many_targ, dm.test_swap, dm.test_pauli_tensor_and_gadget, dm.test_kraus_map, dm.test_channels,
            dm.test_expec_pauli_string, dm.test_partial_trace, dm.test_partial_trace_many_outputs]


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("case", SV_TESTS + DM_TESTS, ids=lambda f: f.__module__[5:] + "." + f.__name__[5:])
def test_wide_index(dfs, oracle, prec, rng, wide, case):
    case(dfs, oracle, prec, rng)


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6])
def test_wide_index_many_targ(dfs, oracle, prec, k, rng, wide):
    sv.test_many_targ(dfs, oracle, prec, k, rng)


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_wide_index_many_targ_6_many_tiles(dfs, oracle, prec, rng, wide):
    sv.test_many_targ_6_many_tiles(dfs, oracle, prec, rng)


def test_wide_index_reductions(dfs, oracle, rng, wide):
    sv.test_reductions_sv(dfs, oracle, rng)


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("case", [adj.test_statevector_gadget_ansatz, adj.test_statevector_gate_mix,
                                  adj.test_density_matrix_channels_and_gadgets],
                         ids=lambda f: f.__name__[5:])
def test_wide_index_adjoint(dfs, oracle, prec, rng, wide, case):
    case(dfs, oracle, prec, rng)


@pytest.mark.parametrize("prec,tol", [("c128", 1e-10), ("c64", 2e-4)])
def test_wide_index_paired_gadgets(dfs, oracle, prec, tol, rng, wide):
    fusion.test_paired_gadgets(dfs, oracle, prec, tol, rng)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_wide_index_noalloc(dfs, prec, wide):
    noalloc.test_noalloc_matches_expecPauliString_twice(dfs, prec)


def test_wide_index_switch_is_restored(dfs, oracle, rng):
    # the fixture turns it off again: the default path still matches
    sv.test_swap(dfs, oracle, "c128", rng)

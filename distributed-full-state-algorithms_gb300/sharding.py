"""Prefix-qubit sharding plans: what each operation exchanges when a state is split over
2^r ranks by its top r qubits.

The reference distributes every state this way (src/states.hpp:32-69): rank p holds the
2^L amplitudes whose top r index bits equal p, L = numQubits - r for a statevector and
2 numQubits - r for a density matrix's vector.  An operation on suffix qubits (below L)
is local; one on a prefix qubit pairs each rank with the rank whose bits differ there and
exchanges all, half, or a packed subset of the amplitudes (src/distributed_statevector.hpp
:18-298, src/distributed_densitymatrix.hpp:15-406, src/communication.hpp:56-177).

This module computes those decisions per rank, as plain data, in the reference's order:
which peer, which amplitudes are sent and where the received ones land, which factors
combine them, and the swaps that move prefix targets into the suffix.  The engine runs on
one GPU per process, so nothing here moves data: a multi-GPU executor would map each
Exchange to one NCCL send/recv pair (or a peer copy into local HBM) and each Local step
to the single-GPU kernel on the local slice.  The plans are checked against the oracle
on CPU shards with the gloo backend (tests/test_sharding_gloo.py).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Sequence

__all__ = [
    "Layout", "Local", "Skip", "Exchange", "Send", "Receive", "AllReduce", "Combine", "Plan",
    "plan_one_targ", "plan_many_ctrl_one_targ", "plan_swap", "plan_many_targ", "plan_pauli",
    "plan_phase_gadget", "plan_dm_unitary", "plan_dm_swap", "plan_dm_pauli", "plan_dm_phase_gadget",
    "plan_dm_kraus", "plan_dm_dephasing", "plan_dm_depolarising", "plan_dm_two_qubit_depolarising",
    "plan_dm_damping", "plan_dm_expec_pauli_string", "plan_dm_partial_trace",
    "reordered_suffix_targets", "non_targeted_qubit_order",
]


def _bit(x: int, b: int) -> int:
    return (x >> b) & 1


@dataclass(frozen=True)
class Layout:
    """One rank's view of a sharded vector: `vec_qubits` = L + r index bits, the top r
    choosing the rank (`rank`), the low L addressing the 2^L local amplitudes."""
    vec_qubits: int
    log_ranks: int
    rank: int

    @property
    def suffix(self) -> int:  # L
        return self.vec_qubits - self.log_ranks

    @property
    def num_local(self) -> int:
        return 1 << self.suffix

    def prefix_bit(self, q: int) -> int:
        """The rank's bit for prefix qubit q (q >= L)."""
        return _bit(self.rank, q - self.suffix)

    def peer(self, *qubits: int) -> int:
        """The rank whose bits differ from this one at the given prefix qubits."""
        p = self.rank
        for q in qubits:
            p ^= 1 << (q - self.suffix)
        return p


# ---------------------------------------------------------------- plan steps

@dataclass(frozen=True)
class Local:
    """The single-rank operation on the local amplitudes (the engine's kernel), with the
    rank's prefix bits where the operation reads global indices (phases, parities)."""
    op: str
    args: tuple = ()


@dataclass(frozen=True)
class Skip:
    """Nothing to do on this rank."""
    reason: str


@dataclass(frozen=True)
class Exchange:
    """Send `count` amplitudes to `peer` and receive as many from it.  `send` names the
    local amplitudes sent: ("all",), ("range", offset), ("bit", qubit, value) -- those
    whose local index has that bit value, in order --, ("ctrls", sorted qubits) -- those
    with all the qubits 1 --, ("bits2", q1, b1, q0, b0), ("depol2_pair", ...) or
    ("buffer",) -- the values the previous step left for sending.  The received ones
    land in a buffer, in the peer's order."""
    peer: int
    count: int
    send: tuple


@dataclass(frozen=True)
class Send:
    """Send `count` amplitudes selected as in Exchange without waiting for a reply."""
    peer: int
    count: int
    send: tuple


@dataclass(frozen=True)
class Receive:
    peer: int
    count: int


@dataclass(frozen=True)
class AllReduce:
    """Sum one complex value over all ranks."""


@dataclass(frozen=True)
class Combine:
    """How local and received amplitudes combine after an exchange (the reference's
    update loop); `kind` names it, `args` holds its factors and selections."""
    kind: str
    args: tuple = ()


@dataclass
class Plan:
    """A sequence of steps for one rank; nested plans (swaps) run in order."""
    steps: list = field(default_factory=list)

    def add(self, *steps) -> "Plan":
        for s in steps:
            if isinstance(s, Plan):
                self.steps.extend(s.steps)
            else:
                self.steps.append(s)
        return self

    @property
    def exchanges(self) -> list:
        return [s for s in self.steps if isinstance(s, (Exchange, Send, Receive, AllReduce))]

    @property
    def communicates(self) -> bool:
        return bool(self.exchanges)


# ---------------------------------------------------------------- statevector

def plan_one_targ(lay: Layout, target: int, gate) -> Plan:
    """distributed_statevector_oneTargGate, src/distributed_statevector.hpp:18-40."""
    if target < lay.suffix:
        return Plan().add(Local("oneTargGate", (target, gate)))
    b = lay.prefix_bit(target)
    return Plan().add(Exchange(lay.peer(target), lay.num_local, ("all",)),
                      Combine("linear", (gate[b][b], gate[b][1 - b])))


def plan_many_ctrl_one_targ(lay: Layout, ctrls: Sequence[int], target: int, gate) -> Plan:
    """distributed_statevector_manyCtrlOneTargGate, src/distributed_statevector.hpp:43-106."""
    prefix = [q for q in ctrls if q >= lay.suffix]
    suffix = sorted(q for q in ctrls if q < lay.suffix)
    if not all(lay.prefix_bit(q) for q in prefix):
        return Plan().add(Skip("a prefix control is 0 on this rank"))
    if target < lay.suffix:
        return Plan().add(Local("manyCtrlOneTargGate", (tuple(suffix), target, gate)))
    if not suffix:
        return plan_one_targ(lay, target, gate)
    b = lay.prefix_bit(target)
    count = lay.num_local >> len(suffix)
    return Plan().add(Exchange(lay.peer(target), count, ("ctrls", tuple(suffix))),
                      Combine("linear_ctrls", (tuple(suffix), gate[b][b], gate[b][1 - b])))


def plan_swap(lay: Layout, q1: int, q2: int) -> Plan:
    """distributed_statevector_swapGate, src/distributed_statevector.hpp:109-187."""
    if q1 > q2:
        q1, q2 = q2, q1
    if q1 == q2:
        return Plan().add(Skip("the same qubit"))
    if q2 < lay.suffix:
        return Plan().add(Local("swapGate", (q1, q2)))
    if q1 >= lay.suffix:
        # whole-rank swap between the ranks whose two bits differ
        if lay.prefix_bit(q1) == lay.prefix_bit(q2):
            return Plan().add(Skip("equal prefix bits: amplitudes stay"))
        return Plan().add(Exchange(lay.peer(q1, q2), lay.num_local, ("all",)), Combine("replace_all"))
    half = lay.num_local // 2
    b2 = lay.prefix_bit(q2)
    peer = lay.peer(q2)
    if q1 == lay.suffix - 1:
        # the half with q1 = !b2 is contiguous: swap it with the peer's
        offset = half * (1 - b2)
        return Plan().add(Exchange(peer, half, ("range", offset)), Combine("replace_range", (offset,)))
    # non-contiguous half: pack the amplitudes with q1 = !b2
    return Plan().add(Exchange(peer, half, ("bit", q1, 1 - b2)), Combine("replace_bit", (q1, 1 - b2)))


def plan_many_targ(lay: Layout, targets: Sequence[int], gate) -> Plan:
    """distributed_statevector_manyTargGate, src/distributed_statevector.hpp:190-224: each
    prefix target is first swapped with the smallest untargeted suffix qubits (in order),
    the gate applied locally, and the swaps undone."""
    if len(targets) > lay.suffix:
        raise ValueError("more targets than suffix qubits")
    mask = 0
    for t in targets:
        mask |= 1 << t
    free = 0
    while _bit(mask, free):
        free += 1
    new = []
    for t in targets:
        if t < lay.suffix:
            new.append(t)
        else:
            new.append(free)
            free += 1
            while _bit(mask, free):
                free += 1
    plan = Plan()
    swaps = [(a, t) for a, t in zip(new, targets) if a != t]
    for a, b in swaps:
        plan.add(plan_swap(lay, a, b))
    plan.add(Local("manyTargGate", (tuple(new), gate)))
    for a, b in swaps:
        plan.add(plan_swap(lay, a, b))
    return plan


def plan_pauli(lay: Layout, targets: Sequence[int], paulis: Sequence[int], gadget: bool, theta: float = 0.0) -> Plan:
    """distributed_statevector_pauliTensorOrGadget, src/distributed_statevector.hpp:227-292:
    the peer differs at the prefix X/Y targets; the suffix X/Y targets flip local indices.
    (A string without X or Y on any qubit is the diagonal operator here, as in the engine
    and the oracle; the reference's loop skips it.)"""
    peer = lay.rank
    mask_xy, mask_yz = 0, 0
    num_y = 0
    for t, p in zip(targets, paulis):
        if p in (1, 2):
            if t >= lay.suffix:
                peer ^= 1 << (t - lay.suffix)
            else:
                mask_xy |= 1 << t
        if p in (2, 3):
            mask_yz ^= 1 << t
        num_y += p == 2
    args = (tuple(targets), tuple(paulis), gadget, theta, mask_xy, mask_yz, num_y)
    if peer == lay.rank:
        return Plan().add(Local("pauliGadget" if gadget else "pauliTensor", args))
    return Plan().add(Exchange(peer, lay.num_local, ("all",)), Combine("pauli", args + (peer,)))


def plan_phase_gadget(lay: Layout, targets: Sequence[int], theta: float) -> Plan:
    """distributed_statevector_phaseGadget, src/distributed_statevector.hpp:295-298: always
    local; the parity reads the rank's prefix bits (src/local_statevector.hpp:138-153)."""
    return Plan().add(Local("phaseGadget", (tuple(targets), theta)))


# ------------------------------------------------------------ density matrix
# A density matrix of n qubits is a 2n-qubit vector (ket bits 0..n-1, bra bits n..2n-1),
# so its layout has vec_qubits = 2n; the unitaries apply the statevector plans to the ket
# and then the bra qubits (src/distributed_densitymatrix.hpp:15-89).

def plan_dm_unitary(lay: Layout, n: int, targets: Sequence[int], gate, conj_gate) -> Plan:
    """distributed_densitymatrix_manyTargGate, src/distributed_densitymatrix.hpp:15-25."""
    return Plan().add(plan_many_targ(lay, targets, gate), plan_many_targ(lay, [t + n for t in targets], conj_gate))


def plan_dm_swap(lay: Layout, n: int, q1: int, q2: int) -> Plan:
    """src/distributed_densitymatrix.hpp:28-33."""
    return Plan().add(plan_swap(lay, q1, q2), plan_swap(lay, q1 + n, q2 + n))


def plan_dm_pauli(lay: Layout, n: int, targets, paulis, gadget: bool, theta: float = 0.0) -> Plan:
    """src/distributed_densitymatrix.hpp:36-63: ket, bra (theta negated for an even number
    of Ys), and a negation of the tensor for an odd number of Ys."""
    odd = sum(p == 2 for p in paulis) % 2 == 1
    bra = [t + n for t in targets]
    plan = Plan().add(plan_pauli(lay, targets, paulis, gadget, theta),
                      plan_pauli(lay, bra, paulis, gadget, theta if (odd or not gadget) else -theta))
    if not gadget and odd:
        plan.add(Local("negate"))
    return plan


def plan_dm_phase_gadget(lay: Layout, n: int, targets, theta: float) -> Plan:
    """src/distributed_densitymatrix.hpp:66-76."""
    return Plan().add(plan_phase_gadget(lay, targets, theta), plan_phase_gadget(lay, [t + n for t in targets], -theta))


def plan_dm_kraus(lay: Layout, n: int, targets, superop) -> Plan:
    """src/distributed_densitymatrix.hpp:79-89: the superoperator on targets ++ targets + n."""
    return plan_many_targ(lay, list(targets) + [t + n for t in targets], superop)


def plan_dm_dephasing(lay: Layout, n: int, qubits: Sequence[int], prob: float) -> Plan:
    """src/distributed_densitymatrix.hpp:90-99: local (the bra bits may be prefix bits)."""
    return Plan().add(Local("dephasing", (tuple(qubits), prob)))


def plan_dm_depolarising(lay: Layout, n: int, q: int, prob: float) -> Plan:
    """distributed_densitymatrix_oneQubitDepolarising, src/distributed_densitymatrix.hpp
    :102-144: with the bra qubit q + n in the prefix, the half of local elements whose ket
    bit q equals the rank's bra bit is exchanged with the peer, then mixed."""
    c1, c2, c3 = 2 * prob / 3, 1 - 2 * prob / 3, 1 - 4 * prob / 3
    if q < n - lay.log_ranks:
        return Plan().add(Local("oneQubitDepolarising", (q, prob)))
    b = lay.prefix_bit(q + n)
    return Plan().add(Exchange(lay.peer(q + n), lay.num_local // 2, ("bit", q, b)),
                      Combine("depol1", (q, b, c1, c2, c3)))


def plan_dm_two_qubit_depolarising(lay: Layout, n: int, q1: int, q2: int, prob: float,
                                   reference_compat: bool = False) -> Plan:
    """twoQubitDepolarising with the reference's branches and exchange volumes
    (src/distributed_densitymatrix.hpp:147-257): local when both bra qubits are suffix
    qubits; "pair" (one exchange of an eighth) when only q2 + n is a prefix qubit; "quad"
    (two exchanges of a quarter) when both are.  Every element whose ket and bra bits of
    q1 and q2 are not both equal is scaled by 1 - 16p/15; each of the four fully diagonal
    elements of a group becomes w x + (4p/15) (their sum), w = 1 - 16p/15 (the
    trace-preserving channel, the engine's default) or 1 - 4p/5 (reference_compat: the
    reference's local loop, src/local_densitymatrix.hpp:83-108).  The sum is formed across
    ranks: pair ranks exchange the sums of their two diagonal elements, quad ranks add
    theirs in two rounds (recursive doubling).  (The reference's own pair and quad loops do
    not reproduce its local loop: the pair update leaves the element itself out of the sum
    and uses the already-updated partner, the quad update keeps only the second partner's
    value; the plan follows the single-rank result.)"""
    if q1 > q2:
        q1, q2 = q2, q1
    w = 1 - 4 * prob / 5 if reference_compat else 1 - 16 * prob / 15
    c2, c3 = 4 * prob / 15, -16 * prob / 15
    threshold = n - lay.log_ranks
    name = "twoQubitDepolarising_referenceCompat" if reference_compat else "twoQubitDepolarising"
    if q2 < threshold:
        return Plan().add(Local(name, (q1, q2, prob)))
    if q1 < threshold:
        # pair: q2 + n in the prefix, q1 + n in the suffix; per group the two diagonal
        # elements here (ket q2 = this rank's bra bit) and two on the peer
        q0, qq1, qq2 = q1, q2, q1 + n
        b = lay.prefix_bit(q2 + n)
        return Plan().add(Combine("depol2_pair_scale", (q0, qq1, qq2, b, c3)),
                          Exchange(lay.peer(q2 + n), lay.num_local // 8, ("depol2_pair", q0, qq1, qq2, b)),
                          Combine("depol2_pair", (q0, qq1, qq2, b, w, c2)))
    # quad: both bra bits in the prefix; each of the four ranks of a group holds one
    # diagonal element per group (ket bits equal to its bra bits)
    b0, b1 = lay.prefix_bit(q1 + n), lay.prefix_bit(q2 + n)
    return Plan().add(Combine("depol2_quad_scale", (q1, q2, b0, b1, c3)),
                      Exchange(lay.peer(q1 + n), lay.num_local // 4, ("bits2", q2, b1, q1, b0)),
                      Combine("depol2_quad_sum", (q1, q2, b0, b1)),
                      Exchange(lay.peer(q2 + n), lay.num_local // 4, ("buffer",)),
                      Combine("depol2_quad_mix", (q1, q2, b0, b1, w, c2)))


def plan_dm_damping(lay: Layout, n: int, q: int, prob: float) -> Plan:
    """distributed_densitymatrix_damping, src/distributed_densitymatrix.hpp:260-319: ranks
    with bra bit 1 send their half (ket bit 1) without waiting; ranks with bra bit 0
    receive it and add p times it to their (ket 0, bra 0) elements."""
    if q < n - lay.log_ranks:
        return Plan().add(Local("damping", (q, prob)))
    b = lay.prefix_bit(q + n)
    peer = lay.peer(q + n)
    half = lay.num_local // 2
    if b == 1:
        return Plan().add(Send(peer, half, ("bit", q, 1)), Combine("damping_sender", (q, prob)))
    return Plan().add(Receive(peer, half), Combine("damping_receiver", (q, prob)))


def plan_dm_expec_pauli_string(lay: Layout, n: int, coeffs, all_paulis) -> Plan:
    """distributed_densitymatrix_expecPauliString, src/distributed_densitymatrix.hpp:322-344:
    a local partial sum over the rank's elements (global indices) and one all-reduce."""
    return Plan().add(Local("expecPauliString_partial", (tuple(coeffs), tuple(all_paulis))), AllReduce())


def _next_leftmost_zero(mask: int, below: int) -> int:
    b = below - 1
    while _bit(mask, b):
        b -= 1
    return b


def reordered_suffix_targets(targets: Sequence[int], suffix: int) -> list[int]:
    """getReorderedAllSuffixTargets, src/misc.hpp:84-104: each prefix target (from the
    last) takes the largest untargeted suffix qubit not yet taken."""
    mask = 0
    for t in targets:
        mask |= 1 << t
    nxt = _next_leftmost_zero(mask, suffix)
    out = []
    for t in reversed(targets):
        if t < suffix:
            out.append(t)
        else:
            out.append(nxt)
            nxt = _next_leftmost_zero(mask, nxt)
    return out[::-1]


def non_targeted_qubit_order(num_all: int, original: Sequence[int], reordered: Sequence[int]) -> list[int]:
    """getNonTargetedQubitOrder, src/misc.hpp:107-133: where each remaining qubit sits
    after the swaps, renumbered contiguously."""
    allq = list(range(num_all))
    for a, b in zip(original, reordered):
        if a != b:
            allq[a], allq[b] = allq[b], allq[a]
    rmask = 0
    for q in reordered:
        rmask |= 1 << q
    remaining = [allq[i] for i in range(num_all) if not _bit(rmask, i)]
    remmask = 0
    for q in remaining:
        remmask |= 1 << q
    return [q - sum(1 for i in range(q) if not _bit(remmask, i)) for q in remaining]


def plan_dm_partial_trace(lay: Layout, n: int, targets: Sequence[int]) -> tuple[Plan, Plan, Plan]:
    """distributed_densitymatrix_partialTrace, src/distributed_densitymatrix.hpp:347-406.
    Returns (swaps on the input, the local trace, reordering swaps on the output, whose
    layout is that of an (n - k)-qubit matrix on the same ranks)."""
    targets = sorted(targets)
    k = len(targets)
    if n - k < lay.log_ranks:
        raise ValueError("the reduced matrix has fewer columns than ranks")
    out_lay = Layout(2 * (n - k), lay.log_ranks, lay.rank)
    if targets and targets[-1] + n < lay.suffix:
        pairs = [t + n for t in targets]
        return Plan(), Plan().add(Local("partialTrace", (tuple(targets), tuple(pairs)))), Plan()
    ext = targets + [t + n for t in targets]
    reo = reordered_suffix_targets(ext, lay.suffix)
    pre = Plan()
    for q in reversed(range(len(reo))):
        if reo[q] != ext[q]:
            pre.add(plan_swap(lay, reo[q], ext[q]))
    trace = Plan().add(Local("partialTrace", (tuple(targets), tuple(reo[k:]))))
    rem = non_targeted_qubit_order(2 * n, ext, reo)
    post = Plan()
    for q in reversed(range(len(rem))):
        if rem[q] == q:
            continue
        p = rem.index(q)
        post.add(plan_swap(out_lay, q, p))
        rem[q], rem[p] = rem[p], rem[q]
    return pre, trace, post

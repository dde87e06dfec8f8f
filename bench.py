"""Benchmark of the GB300 full-state engine (one JSON line on stdout).

Workload: a 30-qubit complex128 statevector (16 GiB, seeded N(0,1) amplitudes,
normalised) driven through a seeded 200-gate circuit drawn uniformly from the
statevector gate mix (one-target Haar 2x2, two-control one-target, swap,
three-target Haar 8x8, Pauli gadgets of weight 2..4, phase gadgets on 2..3
qubits).  A step applies the whole circuit once; the metric is gates/s.  The
end-to-end figure (``e2e``) moves each step's 16 GiB input state up from pinned
host memory and its result back, as a serving loop that overlaps those transfers
with the neighbouring steps' gates (``e2e_blocking``: the same without overlap).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``--impl reference`` times the reference's own CPU code (built from its sources
into oracle/_ref by ``__graft_entry__.build()``; the C restatement in oracle/
when that is unavailable) on the host cores, on a bounded sample of the same
circuit per step.  Under torchrun each rank drives one GPU with its own replica
of the state (the path does not shard: replicas only); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "gates/s & HBM GB/s vs 8 TB/s @30q; adjoint grad/forward ratio; FP32 vs FP64 speedup"
WORKLOAD = "sv30_c128_gate_mix"
NUM_QUBITS = 30
NUM_GATES = 200
CIRCUIT_SEED = 20240611
STATE_SEED = 77
# differentiation form: 24-qubit ansatz of 20 layers x 24 Pauli gadgets, H of 100 terms
ADJ_QUBITS, ADJ_LAYERS, ADJ_PER_LAYER, ADJ_TERMS = 24, 20, 24, 100
# and its density-matrix variant: 11 qubits, the same layers with channels, H of 40 terms
ADJ_DM_QUBITS, ADJ_DM_TERMS = 11, 40
# batched form: 512 circuits of 10..22 qubits, 50 gates each, H of 32 terms
BATCH_CIRCUITS, BATCH_MIN_Q, BATCH_MAX_Q, BATCH_GATES, BATCH_TERMS, BATCH_SEED = 512, 10, 22, 50, 32, 2024
# precision form: 32 qubits, the gate mix plus dense k = 2, 4, 5, 6 gates, H of 100 terms
PREC_QUBITS, PREC_TERMS, PREC_DENSE = 32, 100, (2, 4, 5, 6)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--qubits", type=int, default=NUM_QUBITS)
    ap.add_argument("--gates", type=int, default=NUM_GATES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the e2e, FP32 and native-FP64 legs")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the adjoint, batched and 32-qubit precision legs")
    ap.add_argument("--legs", default="adjoint,batched,precision32,fusion,dm12,dm15",
                    help="comma-separated forms to run (adjoint, batched, precision32, fusion, dm12, dm15)")
    ap.add_argument("--form-scale", default="full", choices=["full", "small"],
                    help="small: the forms at reduced sizes, for profiling captures")
    ap.add_argument("--batch-shape", default=None,
                    help="CTAS_PER_SM,TEAM_WIDTH for the batched leg instead of autotuning")
    return ap.parse_args()


def load_modules():
    import __graft_entry__ as ge
    dfs = ge.package()
    circuits = sys.modules.get("dfs_gb300.circuits")
    if circuits is None:
        import importlib
        circuits = importlib.import_module("dfs_gb300.circuits")
    return dfs, circuits


# ----------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        sm, smax, reasons = [], 0.0, set()
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------- distributed bits

def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_throughput(local_ms: float, units_per_rank: int, world: int, device="cpu") -> tuple[float, float]:
    """Whole-job throughput of independent replicas: every rank processed
    `units_per_rank` units; the job took as long as the slowest rank.
    Returns (units per second over all ranks, max elapsed ms)."""
    ms = local_ms
    if world > 1:
        import torch
        import torch.distributed as td
        t = torch.tensor([local_ms], dtype=torch.float64, device=device)
        td.all_reduce(t, op=td.ReduceOp.MAX)
        ms = float(t.item())
    return world * units_per_rank / (ms / 1e3), ms


def any_rank(flag: bool, world: int) -> bool:
    """Whether `flag` holds on any rank (so that every rank takes the same branch)."""
    if world == 1:
        return flag
    import torch
    import torch.distributed as td
    t = torch.tensor([1.0 if flag else 0.0], dtype=torch.float64, device="cuda")
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item()) > 0


def roofline_traffic(kind: str, qubits: int):
    """DRAM read+write bytes per launch of `kind` (ncu, profiles/traffic.json), scaled from
    the capture's state size to this one; None without a capture of that kind."""
    f = ROOT / "profiles" / "traffic.json"
    try:
        t = json.loads(f.read_text())
        return float(t["bytes_per_launch_at_capture"][kind]) * 2.0 ** (qubits - int(t["capture_qubits"]))
    except (OSError, KeyError, ValueError):
        return None


def measured_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


# ------------------------------------------------------- reference arm

def kinds_of(gates):
    """The circuit's gates by kind, in circuit order."""
    by_kind = {}
    for g in gates:
        by_kind.setdefault(g.kind, []).append(g)
    return by_kind


def reference_sample(run_gate, gates, steps, warmup):
    """Times the reference on a stratified sample of the circuit: step i runs the i-th
    gate of every kind the circuit holds (cyclically, in circuit order), so each step
    covers the whole mix.  The circuit's rate is its gate count over
    sum_kind count_kind * mean_seconds_kind.  Returns (gates/s, details)."""
    by_kind = kinds_of(gates)
    secs = {k: [] for k in by_kind}
    t_steps = []
    for s in range(warmup + steps):
        t_step = 0.0
        for kind, gs in by_kind.items():
            g = gs[s % len(gs)]
            t0 = time.perf_counter()
            run_gate(g)
            dt = time.perf_counter() - t0
            if s >= warmup:
                secs[kind].append(dt)
                t_step += dt
        if s >= warmup:
            t_steps.append(t_step)
    counts = {k: len(v) for k, v in by_kind.items()}
    mean = {k: statistics.fmean(v) for k, v in secs.items()}
    full = sum(counts[k] * mean[k] for k in counts)
    details = {
        "sample": f"stratified: each step runs one gate of each of the {len(counts)} kinds of the "
                  f"{len(gates)}-gate circuit (the i-th of its kind at step i)",
        "kind_counts": counts,
        "kind_seconds": mean,
        "sampled_gates": sum(len(v) for v in secs.values()),
        "sampled_seconds": sum(t_steps),
        "seconds_per_sampled_step": statistics.fmean(t_steps),
        "full_circuit_s_extrapolated": full,
    }
    return len(gates) / full, details


def reference_backend(circuits, n):
    """The reference build (oracle/_ref) with the seeded state, else the C restatement."""
    from oracle.oracle import Oracle, Reference
    amps = seeded_host_state(n, STATE_SEED)
    try:
        backend = Reference()
        h = backend.new_state(amps, False)
        del amps

        def run_gate(g):
            run_reference_gate(backend, h, g)

        return "reference", run_gate, lambda: backend.free_state(h, False)
    except Exception:
        orc = Oracle()

        def run_port(g):
            circuits.apply_to(orc, amps, [g])

        return "port", run_port, lambda: None


def reference_arm(args, circuits):
    """The reference's CPU implementation on the host cores, same workload: the same
    30-qubit seeded state and 200-gate circuit, timed on a stratified sample of it."""
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    os.environ.setdefault("OMP_PROC_BIND", "true")
    os.environ.setdefault("OMP_WAIT_POLICY", "active")
    n = args.qubits
    gates = circuits.gate_mix(n, args.gates, CIRCUIT_SEED)
    kind, run_gate, free = reference_backend(circuits, n)
    value, det = reference_sample(run_gate, gates, args.steps, args.warmup)
    free()
    threads = int(os.environ["OMP_NUM_THREADS"])
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "gates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": det["seconds_per_sampled_step"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "qubits": n, "gates_per_step": len(det["kind_counts"]),
                   "circuit_gates": len(gates), "circuit_seed": CIRCUIT_SEED, "precision": "c128",
                   "state": "seeded N(0,1), normalised", "sample": det["sample"]},
        "reference_timing": det,
        "cpu_baseline": {"value": value, "unit": "gates/s", "cores": threads, "kind": kind,
                         "sample": det["sample"] + f", {args.steps} timed steps, {n} qubits"},
        "e2e": {"value": value, "unit": "gates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference_gate(ref, h, g):
    import ctypes as C
    L = ref.lib

    def u(xs):
        xs = list(xs)
        return (C.c_uint * max(1, len(xs)))(*xs), len(xs)

    if g.kind in ("one_targ", "ctrl", "many_targ"):
        m = np.ascontiguousarray(g.matrix, dtype=np.complex128)
        mp = m.ctypes.data_as(C.c_void_p)
    if g.kind == "one_targ":
        L.ref_sv_one_targ(h, g.qubits[0], mp)
    elif g.kind == "ctrl":
        c, nc = u(g.controls)
        L.ref_sv_many_ctrl_one_targ(h, c, nc, g.qubits[0], mp)
    elif g.kind == "swap":
        L.ref_sv_swap(h, g.qubits[0], g.qubits[1])
    elif g.kind == "many_targ":
        t, k = u(g.qubits)
        L.ref_sv_many_targ(h, t, k, mp)
    elif g.kind == "pauli_gadget":
        t, k = u(g.qubits)
        p, _ = u(g.paulis)
        L.ref_sv_pauli_gadget(h, t, p, k, g.param)
    elif g.kind == "phase_gadget":
        t, k = u(g.qubits)
        L.ref_sv_phase_gadget(h, t, k, g.param)
    else:
        raise ValueError(g.kind)


def seeded_host_state(n, seed):
    """N(0,1) real and imaginary parts, normalised, generated on the host in
    parallel chunks (numpy releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    N = 1 << n
    out = np.empty(N, dtype=np.complex128)
    view = out.view(np.float64)
    chunks = max(1, min(64, N >> 20))
    seqs = np.random.SeedSequence(seed).spawn(chunks)
    step = (2 * N) // chunks

    def fill(i):
        np.random.default_rng(seqs[i]).standard_normal(out=view[i * step:(i + 1) * step])
        return float(np.dot(view[i * step:(i + 1) * step], view[i * step:(i + 1) * step]))

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        total = sum(ex.map(fill, range(chunks)))
    out *= 1.0 / np.sqrt(total)
    return out


# ------------------------------------------------------------- GPU arm

def gpu_arm(args, world, rank, local):
    import torch
    dfs, circuits = load_modules()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as td
        td.init_process_group("nccl", device_id=torch.device("cuda", local))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dfs.comm_init()
    dfs.set_stream(stream)
    n = args.qubits
    gates = circuits.gate_mix(n, args.gates, CIRCUIT_SEED)
    elem = 16
    num_amps = 1 << n

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as td
            td.barrier()

    psi = dfs.StateVector(n, precision="c128")
    psi.setRandomAmps(seed=STATE_SEED, normalise=True)

    # warm-up
    for _ in range(args.warmup):
        circuits.apply(dfs, psi, gates)

    # timed region: per-gate events on the engine stream for the kernel breakdown
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(len(gates) * args.steps)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    start.record(stream)
    i = 0
    for _ in range(args.steps):
        for g in gates:
            evs[i][0].record(stream)
            circuits.apply(dfs, psi, [g])
            evs[i][1].record(stream)
            i += 1
    stop.record(stream)
    barrier()
    clock_info = clocks.stop()
    total_gates = len(gates) * args.steps
    value, elapsed_ms = replica_throughput(start.elapsed_time(stop), total_gates, world, device="cuda")

    per_kind = {}
    for j, (a, b) in enumerate(evs):
        g = gates[j % len(gates)]
        d = per_kind.setdefault(g.kind, {"ms": 0.0, "launches": 0, "bytes": 0})
        d["ms"] += a.elapsed_time(b)
        d["launches"] += circuits.kernel_launches(g)
        d["bytes"] += circuits.algorithmic_bytes(g, num_amps, elem)
    kernel_ms = sum(d["ms"] for d in per_kind.values())
    kernels = {}
    for kind, d in per_kind.items():
        kernels[kind] = {"launches": d["launches"], "ms_avg": d["ms"] / d["launches"],
                         "share": d["ms"] / kernel_ms, "gbs": d["bytes"] / (d["ms"] * 1e-3) / 1e9}
    dominant = max(kernels, key=lambda k: kernels[k]["share"])
    peak, peak_kind = measured_peak()
    dom_bytes = per_kind[dominant]["bytes"] / per_kind[dominant]["launches"]
    achieved = kernels[dominant]["gbs"]
    all_bytes = sum(d["bytes"] for d in per_kind.values())
    algo_gbs = all_bytes / (elapsed_ms * 1e-3) / 1e9

    result = {
        "metric": METRIC, "value": value, "unit": "gates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "arith": "IEEE f64 storage; double-float (2 x f32, >= 47-bit) arithmetic on the FP32 pipes",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "qubits": n, "gates_per_step": len(gates), "precision": "c128",
                   "circuit_seed": CIRCUIT_SEED, "state": "seeded N(0,1), normalised, device generator",
                   "l2": "state 16 GiB > L2 129 MB: no flush needed", "parallelism": f"replicas x{world}"},
        "hbm_gbs_algorithmic": algo_gbs,
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": roofline_traffic(dominant, n), "algorithmic_bytes_per_launch": dom_bytes},
        "kernels": kernels,
        "gpu_launches": sum(d["launches"] for d in per_kind.values()),
        "clocks": clock_info,
    }

    if not args.no_extras:
        import ctypes as C
        lib = dfs.load_library()
        hosts = [torch.empty(num_amps * 2, dtype=torch.float64, pin_memory=True)]
        psi2 = None
        try:  # the serving loop's pinned input and output buffers (two each) and second state
            for _ in range(3):
                hosts.append(torch.empty(num_amps * 2, dtype=torch.float64, pin_memory=True))
            psi2 = dfs.StateVector(n)
        except (RuntimeError, dfs.DfsError):
            pass
        serving = not any_rank(psi2 is None, world)
        for h in hosts:  # valid input states
            assert lib.dfs_state_get_raw(psi.handle, C.c_void_p(h.data_ptr()), 0, num_amps) == 0
        # the serving loop runs as many steps as the timed region (at least 2); the blocking
        # loop, a diagnostic of the transfer phases when the serving loop runs, takes 3
        e2e_steps = max(2, args.steps)
        blocking_steps = min(3, e2e_steps) if serving else e2e_steps
        # end to end through the public API with host buffers, as a blocking loop: upload
        # the step's input state from pinned memory, run the circuit, read it back
        ptr = C.c_void_p(hosts[0].data_ptr())
        barrier()
        t0 = time.perf_counter()
        phases = []  # per step: upload, circuit, download (each call ends synchronised)
        for _ in range(blocking_steps):
            ta = time.perf_counter()
            assert lib.dfs_state_set_raw(psi.handle, ptr, 0, num_amps) == 0
            tb = time.perf_counter()
            circuits.apply(dfs, psi, gates)
            dfs.comm_synch()
            tc = time.perf_counter()
            assert lib.dfs_state_get_raw(psi.handle, ptr, 0, num_amps) == 0
            phases.append((tb - ta, tc - tb, time.perf_counter() - tc))
        barrier()
        blocking_s = time.perf_counter() - t0
        per_step = {"h2d_bytes_per_step": num_amps * elem, "d2h_bytes_per_step": num_amps * elem}
        med = [statistics.median(ph[j] for ph in phases) for j in range(3)]
        blocking = {"value": world * len(gates) * blocking_steps / blocking_s, "unit": "gates/s", **per_step,
                    "mode": f"{blocking_steps} steps of upload, circuit, download in turn",
                    "median_s": {"upload": med[0], "circuit": med[1], "download": med[2]},
                    "host_link_gbs": {"h2d": num_amps * elem / med[0] / 1e9, "d2h": num_amps * elem / med[2] / 1e9}}
        if serving:
            # the same as a serving loop: the transfers go on the engine's copy streams
            # (dfs_state_set_raw_async / get_raw_async, one stream per direction), so step
            # i+1's upload and step i-1's download overlap step i's gates and each other; two
            # device states, two pinned input buffers and two pinned output buffers
            ins, outs = hosts[:2], hosts[2:]
            states = [psi, psi2]
            barrier()
            t0 = time.perf_counter()
            states[0].uploadAsync(ins[0])
            for i in range(e2e_steps):
                cur, nxt = states[i % 2], states[(i + 1) % 2]
                if i + 1 < e2e_steps:
                    nxt.uploadAsync(ins[(i + 1) % 2])
                circuits.apply(dfs, cur, gates)
                cur.downloadAsync(outs[i % 2])
            for st in states:
                st.waitTransfers()
            dfs.comm_synch()
            barrier()
            e2e_s = time.perf_counter() - t0
            result["e2e"] = {"value": world * len(gates) * e2e_steps / e2e_s, "unit": "gates/s", **per_step,
                             "mode": f"serving loop of {e2e_steps} steps, transfers overlapped on two copy streams"}
            result["e2e_blocking"] = blocking
        else:  # no room for a second state or pinned buffer on some rank
            result["e2e"] = blocking
        del hosts
        psi.free()
        if psi2 is not None:
            psi2.free()

        # FP32 form: the same circuit on a complex64 state
        phi = dfs.StateVector(n, precision="c64")
        phi.setRandomAmps(seed=STATE_SEED, normalise=True)
        circuits.apply(dfs, phi, gates)
        barrier()
        t0 = time.perf_counter()
        f32_steps = max(1, min(3, args.steps))
        for _ in range(f32_steps):
            circuits.apply(dfs, phi, gates)
        barrier()
        f32 = len(gates) * f32_steps / (time.perf_counter() - t0)
        phi.free()
        # native FP64 arithmetic: the same circuit, IEEE double FMA (1.2 TFLOP/s on GB300)
        nat = dfs.StateVector(n, precision="c128_native")
        nat.setRandomAmps(seed=STATE_SEED, normalise=True)
        circuits.apply(dfs, nat, gates[:20])
        barrier()
        t0 = time.perf_counter()
        circuits.apply(dfs, nat, gates)
        barrier()
        native = len(gates) / (time.perf_counter() - t0)
        nat.free()
        per_gpu = value / world
        result["fp32"] = {"gates_per_s": f32, "speedup_vs_f64": f32 / per_gpu}
        result["f64_native"] = {"gates_per_s": native, "emulated_speedup": per_gpu / native}
    else:
        psi.free()

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args, circuits, gates)
    if not args.no_forms:
        legs = {"adjoint": adjoint_leg, "batched": batch_leg, "precision32": precision_leg, "fusion": fusion_leg,
                "dm12": dm_leg, "dm15": dm_kernels_leg}
        for name in [x for x in args.legs.split(",") if x]:
            if name not in legs:
                result[name] = {"error": "unknown leg"}
                continue
            try:
                result[name] = legs[name](dfs, circuits, small=args.form_scale == "small")
            except Exception as e:  # a failing extra leg must not lose the headline line
                result[name] = {"error": f"{type(e).__name__}: {e}"}
    return result, rank


# ------------------------------------------------- forms beyond plain FP64

def _sync_time(dfs, fn):
    dfs.comm_synch()
    t0 = time.perf_counter()
    out = fn()
    dfs.comm_synch()
    return (time.perf_counter() - t0) * 1e3, out


def adjoint_leg(dfs, circuits, small=False):
    """Full adjoint gradient against one forward pass (same <H>), complex128 and complex64."""
    n = ADJ_QUBITS  # already a few-GB case (two 256 MiB vectors)
    gates = circuits.gadget_ansatz(n, ADJ_LAYERS, ADJ_PER_LAYER, seed=CIRCUIT_SEED)
    coeffs, paulis = circuits.pauli_sum(n, ADJ_TERMS, seed=7)
    circ, params = circuits.record(dfs, n, gates)
    out = {"workload": f"sv{n} ansatz {ADJ_LAYERS}x{ADJ_PER_LAYER} Pauli gadgets ({params.size} parameters), "
                       f"H of {ADJ_TERMS} terms; forward = circuit + H psi + <H>; gradient = forward + backward"}
    grads = {}
    for prec in ("c128", "c64"):
        init = dfs.StateVector(n, precision=prec)
        init.setRandomAmps(seed=STATE_SEED, normalise=True)
        circ.expectation(init, params, coeffs, paulis)
        circ.gradient(params)
        fw, bw, plain = [], [], []
        work = dfs.StateVector(n, precision=prec)
        for _ in range(3):
            fw.append(_sync_time(dfs, lambda: circ.expectation(init, params, coeffs, paulis))[0])
            ms, grads[prec] = _sync_time(dfs, lambda: circ.gradient(params))
            bw.append(ms)
            work.copyFrom(init)
            plain.append(_sync_time(dfs, lambda: (circ.apply(work, params),
                                                  dfs.statevector_expecPauliSum(work, coeffs, paulis)))[0])
        f, b, p = statistics.median(fw), statistics.median(bw), statistics.median(plain)
        out[prec] = {"forward_ms": f, "backward_ms": b, "gradient_over_forward": (f + b) / f,
                     "gradient_over_plain_forward": (f + b) / p, "plain_forward_ms": p}
        init.free()
        work.free()
    scale = float(np.max(np.abs(grads["c128"])))
    out["c64_gradient_max_rel_err"] = float(np.max(np.abs(grads["c64"] - grads["c128"]))) / scale
    # the density-matrix variant: 11 qubits, the gadgets' angles and the depolarising and
    # damping probabilities as parameters (checkpoints before the channels)
    nd = ADJ_DM_QUBITS
    dgates = circuits.dm_gadget_ansatz(nd, ADJ_LAYERS, ADJ_PER_LAYER, seed=CIRCUIT_SEED)
    dcoeffs, dpaulis = circuits.pauli_sum(nd, ADJ_DM_TERMS, seed=12)
    dcirc, dparams = circuits.record(dfs, nd, dgates, density_matrix=True)
    rng = np.random.default_rng(4)
    g = rng.normal(size=(1 << nd, 1 << nd)) + 1j * rng.normal(size=(1 << nd, 1 << nd))
    rho = g @ g.conj().T
    rho /= np.trace(rho).real
    init = dfs.DensityMatrix(nd)
    init.setMatrix(rho)
    dcirc.expectation(init, dparams, dcoeffs, dpaulis)
    dcirc.gradient(dparams)
    fw, bw = [], []
    for _ in range(3):
        fw.append(_sync_time(dfs, lambda: dcirc.expectation(init, dparams, dcoeffs, dpaulis))[0])
        bw.append(_sync_time(dfs, lambda: dcirc.gradient(dparams))[0])
    f, b = statistics.median(fw), statistics.median(bw)
    out["dm_c128"] = {"workload": f"dm{nd} ansatz {ADJ_LAYERS} x ({ADJ_PER_LAYER} Pauli gadgets + depolarising + "
                                  f"damping), {dparams.size} parameters, H of {ADJ_DM_TERMS} terms",
                      "forward_ms": f, "backward_ms": b, "gradient_over_forward": (f + b) / f}
    init.free()
    dcirc.free()
    return out


def batch_bytes(specs, circuits, elem):
    """Algorithmic bytes of one batched run with gradients: the initial-state copy, each
    gate, H psi (T reads, the loss read, one write), and each gate's backward step (the
    state and the adjoint)."""
    total = 0
    for n, gates, coeffs, _ in specs:
        N = 1 << n
        total += 2 * N * elem + (len(coeffs) + 2) * N * elem
        for g in gates:
            fb = circuits.algorithmic_bytes(g, N, elem)
            total += fb + 2 * fb
    return total


BATCH_SHAPE = None  # (CTAs per SM, team width) from --batch-shape


def batch_leg(dfs, circuits, small=False):
    """One persistent launch (graph replay) for every circuit's <H> and gradient, against
    per-circuit runs through the circuit runtime."""
    specs = circuits.batch_mix(128 if small else BATCH_CIRCUITS, BATCH_MIN_Q, BATCH_MAX_Q, BATCH_GATES, BATCH_TERMS,
                               BATCH_SEED)
    recs = [circuits.record(dfs, n, g, parametrise=("pauli_gadget", "phase_gadget")) for n, g, _, _ in specs]
    circs = [r[0] for r in recs]
    params = [r[1] for r in recs]
    out = {"workload": f"{len(specs)} statevector circuits of {BATCH_MIN_Q}-{max(x[0] for x in specs)} qubits, "
                       f"{BATCH_GATES} gates each, H of {BATCH_TERMS} terms, <H> and adjoint gradient per circuit",
           "total_amplitudes": int(sum(1 << s[0] for s in specs))}
    for prec, elem in (("c128", 16), ("c64", 8)):
        b = dfs.Batch(circs, precision=prec)
        for i, (n, _, c, p) in enumerate(specs):
            b.setHamiltonian(i, c, p)
        b.setRandomStates(seed=STATE_SEED)
        b.setParams(np.concatenate(params))
        t0 = time.perf_counter()
        if BATCH_SHAPE:
            b.setShape(*BATCH_SHAPE)
        else:
            b.autotune(gradient=True)
        tune_s = time.perf_counter() - t0
        b.run(gradient=True)
        runs = [_sync_time(dfs, lambda: b.run(gradient=True))[0] for _ in range(3)]
        batch_ms = statistics.median(runs)
        cps, width = b.shape
        b.free()
        inits = []
        for i, (n, _, c, p) in enumerate(specs):
            s0 = dfs.StateVector(n, precision=prec)
            s0.setRandomAmps(seed=STATE_SEED + i, normalise=True)
            inits.append(s0)

        def sequential():
            for i, (n, _, c, p) in enumerate(specs):
                circs[i].expectation(inits[i], params[i], c, p)
                circs[i].gradient(params[i])

        sequential()
        seq_ms = min(_sync_time(dfs, sequential)[0] for _ in range(2))
        for s0 in inits:
            s0.free()
        nbytes = batch_bytes(specs, circuits, elem)
        out[prec] = {"batch_ms": batch_ms, "sequential_ms": seq_ms, "speedup": seq_ms / batch_ms,
                     "shape": {"ctas_per_sm": cps, "team_width": width}, "autotune_s": tune_s,
                     "algorithmic_gb": nbytes / 1e9, "gbs_algorithmic": nbytes / (batch_ms * 1e-3) / 1e9}
    return out


def dense_kernels(dfs, circuits, psi, n):
    """Each complex128 dense gate size alone on an n-qubit state: CUDA-event ms on the engine
    stream (best of 3), algorithmic GB/s (the state read and written once) and fraction of
    the measured copy bandwidth, with the tensor-pipe and ALU-pipe shares of its kernel
    from the one-kernel ncu capture in profiles/dense_tensor_pipe.json."""
    import torch
    peak, peak_kind = measured_peak()
    try:
        prof = json.loads((ROOT / "profiles" / "dense_tensor_pipe.json").read_text())["kernels"]
    except (OSError, KeyError, ValueError):
        prof = {}
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream()
    out = {"qubits": n, "peak_gbs": peak, "peak_kind": peak_kind}
    for k in (2, 3, 4, 5, 6):
        targets = [int(t) for t in rng.choice(n, size=k, replace=False)]
        u = circuits.haar_unitary(rng, 1 << k)
        dfs.distributed_statevector_manyTargGate(psi, targets, u)
        best = None
        for _ in range(3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            dfs.distributed_statevector_manyTargGate(psi, targets, u)
            b.record(stream)
            b.synchronize()
            best = a.elapsed_time(b) if best is None else min(best, a.elapsed_time(b))
        gbs = 2 * (1 << n) * 16 / (best * 1e-3) / 1e9
        entry = {"targets": targets, "ms": best, "gbs": gbs, "frac": gbs / peak}
        entry.update(prof.get(str(k), {}))
        out[f"k{k}"] = entry
    return out


def precision_leg(dfs, circuits, small=False):
    """complex64 against complex128 at 32 qubits: time, <H> error and fidelity; the
    complex128 engine (parity-pinned to the oracle) stands for the FP64 reference."""
    n = 26 if small else PREC_QUBITS
    gates = circuits.gate_mix(n, NUM_GATES, CIRCUIT_SEED, dense_k=PREC_DENSE)
    coeffs, paulis = circuits.pauli_sum(n, PREC_TERMS, seed=7)
    res = {"workload": f"sv{n} gate mix + dense k={list(PREC_DENSE)}, {NUM_GATES} gates, H of {PREC_TERMS} terms"}
    states, expec = {}, {}
    for prec in ("c128", "c64"):
        s0 = dfs.StateVector(n, precision=prec)
        s0.setRandomAmps(seed=STATE_SEED, normalise=True)
        ms, _ = _sync_time(dfs, lambda: circuits.apply(dfs, s0, gates))
        expec[prec] = dfs.statevector_expecPauliSum(s0, coeffs, paulis).real
        res[prec] = {"gates_per_s": len(gates) / (ms * 1e-3), "ms": ms}
        states[prec] = s0
    conv = dfs.StateVector(n, precision="c128")
    conv.copyFrom(states["c64"])
    ip = dfs.inner_product(states["c128"], conv)
    fid = abs(ip) ** 2 / (dfs.norm_squared(states["c128"]) * dfs.norm_squared(conv))
    res["dense_c128"] = dense_kernels(dfs, circuits, states["c128"], n)
    for s0 in list(states.values()) + [conv]:
        s0.free()
    res["c64_speedup"] = res["c64"]["gates_per_s"] / res["c128"]["gates_per_s"]
    res["expec_abs_err"] = abs(expec["c64"] - expec["c128"])
    res["expec_rel_err"] = res["expec_abs_err"] / float(np.sum(np.abs(coeffs)))
    res["fidelity"] = fid
    return res


def fusion_leg(dfs, circuits, small=False):
    """Gate fusion of forward passes through the circuit runtime, against the same circuit
    operation by operation: the gate mix (random qubits: short runs) and a circuit of gates
    on the 11 lowest qubits (long runs)."""
    n = 26 if small else NUM_QUBITS
    res = {"workload": f"sv{n}: gate mix of {NUM_GATES} gates, and {NUM_GATES} gates on the 11 lowest qubits "
                       "(every 20th on any qubit); Circuit.apply with and without fusion"}
    for name, gates in (("gate_mix", circuits.gate_mix(n, NUM_GATES, CIRCUIT_SEED)),
                        ("low_qubit", circuits.low_qubit_mix(n, NUM_GATES, 11, seed=CIRCUIT_SEED))):
        circ, params = circuits.record(dfs, n, gates)
        for prec in ("c128", "c64"):
            psi = dfs.StateVector(n, precision=prec)
            psi.setRandomAmps(seed=STATE_SEED, normalise=True)
            times = {}
            for fusion in (False, True):
                circ.fusion = fusion
                circ.apply(psi, params)
                times[fusion] = _sync_time(dfs, lambda: circ.apply(psi, params))[0]
            runs, fused_ops = circ.fusedRuns(prec)
            res[f"{name}_{prec}"] = {"gates_per_s_fused": len(gates) / (times[True] * 1e-3),
                                     "gates_per_s_unfused": len(gates) / (times[False] * 1e-3),
                                     "speedup": times[False] / times[True], "runs": runs, "fused_ops": fused_ops}
            psi.free()
        circ.free()
    return res


def run_reference_dm_op(ref, h, g):
    import ctypes as C
    L = ref.lib
    if g.kind == "dm_many_targ":
        t = (C.c_uint * len(g.qubits))(*g.qubits)
        m = np.ascontiguousarray(g.matrix, dtype=np.complex128)
        L.ref_dm_many_targ(h, t, len(g.qubits), m.ctypes.data_as(C.c_void_p))
    elif g.kind == "deph1":
        L.ref_dm_deph1(h, g.qubits[0], g.param)
    elif g.kind == "deph2":
        L.ref_dm_deph2(h, g.qubits[0], g.qubits[1], g.param)
    elif g.kind == "depol1":
        L.ref_dm_depol1(h, g.qubits[0], g.param)
    elif g.kind == "depol2":
        L.ref_dm_depol2(h, g.qubits[0], g.qubits[1], g.param)
    elif g.kind == "damping":
        L.ref_dm_damping(h, g.qubits[0], g.param)
    else:
        raise ValueError(g.kind)


def dm_kernels_leg(dfs, circuits, small=False):
    """Every density-matrix kernel on a 15-qubit complex128 matrix (a 30-qubit vector,
    16 GiB, far above L2), each timed with CUDA events on the engine stream: ms per call,
    algorithmic bytes (read + write of the elements the operation can change) per second
    and the fraction of the measured copy bandwidth."""
    import torch
    n = 12 if small else 15
    N, B = 1 << (2 * n), 16
    rng = np.random.default_rng(15)
    peak, peak_kind = measured_peak()
    rho = dfs.DensityMatrix(n)
    rho.setRandomAmps(seed=5, normalise=True)
    u1, u2, u3 = (circuits.haar_unitary(rng, d) for d in (2, 4, 8))
    red1, red3 = dfs.DensityMatrix(n - 1), dfs.DensityMatrix(n - 3)  # partialTrace outputs, reused
    coeffs, paulis = circuits.pauli_sum(n, 16, seed=3)
    p = 0.05
    cases = [
        ("oneQubitDephasing", "Deph1Op (k_pair)", N * B, lambda: dfs.distributed_densitymatrix_oneQubitDephasing(rho, 3, p)),
        ("twoQubitDephasing", "k_deph2", 1.5 * N * B, lambda: dfs.distributed_densitymatrix_twoQubitDephasing(rho, 5, 9, p)),
        ("twoQubitDephasing (qubit 0)", "k_deph2", 1.5 * N * B,
         lambda: dfs.distributed_densitymatrix_twoQubitDephasing(rho, 0, 9, p)),
        ("oneQubitDepolarising", "k_quad<Depol1Op>", 2 * N * B, lambda: dfs.distributed_densitymatrix_oneQubitDepolarising(rho, 5, p)),
        ("twoQubitDepolarising", "k_depol2", 2 * N * B, lambda: dfs.distributed_densitymatrix_twoQubitDepolarising(rho, 1, 11, p)),
        ("damping", "k_quad<DampingOp>", 2 * N * B, lambda: dfs.distributed_densitymatrix_damping(rho, 7, p)),
        ("manyTargGate k=1", "superoperator on 2 targets (tensor cores, as S (x) I on 3)", 2 * N * B,
         lambda: dfs.distributed_densitymatrix_manyTargGate(rho, [4], u1)),
        ("manyTargGate k=2", "superoperator on 4 targets (tensor cores)", 2 * N * B,
         lambda: dfs.distributed_densitymatrix_manyTargGate(rho, [2, 10], u2)),
        ("manyTargGate k=3", "U then conj(U) (two 3-target sweeps)", 4 * N * B,
         lambda: dfs.distributed_densitymatrix_manyTargGate(rho, [0, 6, 12], u3)),
        ("swapGate", "k_dm_swap", 1.5 * N * B, lambda: dfs.distributed_densitymatrix_swapGate(rho, 6, 13)),
        ("swapGate (qubit 0)", "k_dm_swap", 1.5 * N * B, lambda: dfs.distributed_densitymatrix_swapGate(rho, 0, 13)),
        ("pauliTensor", "doubled string (k_pair_raw<PauliTensorOp>)", 2 * N * B,
         lambda: dfs.distributed_densitymatrix_pauliTensor(rho, [1, 6, 8], [1, 2, 3])),
        ("pauliGadget", "k_dm_gadget", 2 * N * B, lambda: dfs.distributed_densitymatrix_pauliGadget(rho, [1, 6, 8], [1, 2, 3], 0.3)),
        ("phaseGadget", "k_diag<DmDiagPhaseOp>", 2 * N * B, lambda: dfs.distributed_densitymatrix_phaseGadget(rho, [3, 9], 0.4)),
        ("expecPauliString (16 terms)", "k_expec_dm", 16 * (1 << n) * B,
         lambda: dfs.distributed_densitymatrix_expecPauliString(rho, coeffs, paulis)),
        ("partialTrace (1 qubit)", "k_partial_trace", (N // 2 + N // 4) * B,
         lambda: dfs.distributed_densitymatrix_partialTrace(rho, [4], out=red1)),
        ("partialTrace (3 qubits)", "k_partial_trace", (N // 8 + N // 64) * B,
         lambda: dfs.distributed_densitymatrix_partialTrace(rho, [0, 7, 13], out=red3)),
    ]
    stream = torch.cuda.current_stream()
    out = {"workload": f"{n}-qubit density matrix, c128 ({N} amplitudes, {N * B / 2**30:.0f} GiB)",
           "peak_gbs": peak, "peak_kind": peak_kind, "kernels": {}}
    for name, kernel, nbytes, fn in cases:
        fn()  # warm-up (and the first call's host set-up)
        times = []
        for _ in range(3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
        ms = statistics.median(times)
        gbs = nbytes / (ms * 1e-3) / 1e9
        out["kernels"][name] = {"kernel": kernel, "ms": ms, "algorithmic_bytes": nbytes, "gbs": gbs,
                                "frac": gbs / peak}
    rho.free()
    red1.free()
    red3.free()
    return out


def dm_leg(dfs, circuits, small=False):
    """The plain FP64 density-matrix workflow at 12 qubits: rho = G G^dagger / tr, 10 layers
    of a 2-target Haar unitary and the five channels, expecPauliString over 64 strings and
    partialTrace over 4 qubits, on the GPU; the reference's CPU code on one layer and one
    string of the same workflow (extrapolated to the whole)."""
    import ctypes as C
    n = 12
    rng = np.random.default_rng(12)
    d = 1 << n
    g = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    rho0 = g @ g.conj().T
    rho0 = (rho0 / np.trace(rho0).real).reshape(-1, order="F").copy()
    del g
    ops = circuits.dm_layers(n, 10, seed=2024, max_prob=0.1)
    coeffs, paulis = circuits.pauli_sum(n, 64, seed=99)
    targets = [int(q) for q in rng.choice(n, 4, replace=False)]
    rho = dfs.DensityMatrix(n)
    rho.setAmps(rho0)
    start = dfs.DensityMatrix(n)
    start.copyFrom(rho)
    res = {"workload": "12-qubit density matrix (2^24 amplitudes, c128): 10 layers x (2-target Haar + 5 channels), "
                       "expecPauliString over 64 strings, partialTrace over 4 qubits"}
    for rep in range(2):  # the first repetition warms up
        rho.copyFrom(start)
        t_layers = _sync_time(dfs, lambda: circuits.apply(dfs, rho, ops))[0]
        t_expec = _sync_time(dfs, lambda: dfs.distributed_densitymatrix_expecPauliString(rho, coeffs, paulis))[0]
        t_pt = _sync_time(dfs, lambda: dfs.distributed_densitymatrix_partialTrace(rho, targets).free())[0]
    res["gpu_ms"] = {"layers": t_layers, "expecPauliString_64": t_expec, "partialTrace": t_pt,
                     "total": t_layers + t_expec + t_pt}
    rho.free()
    start.free()
    try:
        from oracle.oracle import Reference
        ref = Reference()
        h = ref.new_state(rho0, True)
        layer = ops[:6]
        t0 = time.perf_counter()
        for gate in layer:
            run_reference_dm_op(ref, h, gate)
        t_layer = time.perf_counter() - t0
        c1 = np.ascontiguousarray(coeffs[:1])
        p1 = np.ascontiguousarray(paulis[:1].ravel().astype(np.uint32))
        out = np.zeros(2)
        t0 = time.perf_counter()
        ref.lib.ref_dm_expec_pauli_string(h, c1.ctypes.data_as(C.c_void_p), 1, p1.ctypes.data_as(C.c_void_p),
                                          out.ctypes.data_as(C.c_void_p))
        t_term = time.perf_counter() - t0
        tq = (C.c_uint * 4)(*targets)
        red = np.zeros(1 << (2 * (n - 4)), dtype=np.complex128)
        t0 = time.perf_counter()
        ref.lib.ref_dm_partial_trace(h, tq, 4, red.ctypes.data_as(C.c_void_p))
        t_ref_pt = time.perf_counter() - t0
        ref.free_state(h, True)
        total = 10 * t_layer + 64 * t_term + t_ref_pt
        res["reference_cpu"] = {"cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
                                "kind": "reference", "layer_s": t_layer, "expec_term_s": t_term,
                                "partialTrace_s": t_ref_pt, "total_s_extrapolated": total,
                                "sample": "one layer and one Pauli string timed; total = 10 layers + 64 strings"}
        res["speedup_vs_reference"] = total / (res["gpu_ms"]["total"] * 1e-3)
    except Exception as e:  # the reference build is optional here
        res["reference_cpu"] = {"error": f"{type(e).__name__}: {e}"}
    return res


def cpu_baseline(args, circuits, gates):
    """The reference's CPU code (oracle/_ref) on the host cores: the same circuit on the
    same-size state, timed on the stratified sample of reference_sample (three steps after
    one warm-up step: every kind of the mix, about 15-25 s of CPU work)."""
    try:
        kind, run_gate, free = reference_backend(circuits, args.qubits)
    except Exception as e:  # pragma: no cover
        return {"value": None, "error": str(e)}
    value, det = reference_sample(run_gate, gates, 3, 1)
    free()
    cores = os.cpu_count() or 1
    return {"value": value, "unit": "gates/s", "cores": int(os.environ.get("OMP_NUM_THREADS", cores)),
            "kind": kind, "sample": det["sample"] + f", 3 timed steps, {args.qubits} qubits",
            "kind_counts": det["kind_counts"], "kind_seconds": det["kind_seconds"],
            "full_circuit_s_extrapolated": det["full_circuit_s_extrapolated"]}


def main():
    global BATCH_SHAPE
    args = parse()
    if args.batch_shape:
        BATCH_SHAPE = tuple(int(x) for x in args.batch_shape.split(","))
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        if rank != 0:
            return
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        _, circuits = load_modules()
        print(json.dumps(reference_arm(args, circuits)), flush=True)
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    result, rank = gpu_arm(args, world, rank, local)
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()

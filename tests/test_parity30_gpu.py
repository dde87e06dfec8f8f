"""Amplitude-wise parity at the benchmark's own size: the 30-qubit complex128 state and
200-gate circuit of the gate mix (the workload bench.py measures) on the engine and on
the oracle (the C restatement of src/local_statevector.hpp:14-153, OpenMP on every host
core), from the same seeded state, compared on all 2^30 amplitudes at 1e-12 of the
largest, for the default (double-float) and the native-FP64 complex128 forms.

The engine state is read back in chunks, so the host holds the oracle's 16 GiB state
and one chunk.  This takes about a minute of host time (the oracle's 200 sweeps).
"""
import ctypes as C
import os
import time

import numpy as np
import pytest

from adjoint_ref import circuits

pytestmark = pytest.mark.gpu

N_QUBITS = 30
CIRCUIT_SEED = 20240611
CHUNK = 1 << 24


def host_ram_bytes():
    try:
        return os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    except (ValueError, OSError):
        return 0


def seeded_state(n, seed):
    """N(0,1) real and imaginary parts, normalised, made on the host in parallel chunks."""
    from concurrent.futures import ThreadPoolExecutor
    N = 1 << n
    out = np.empty(N, dtype=np.complex128)
    view = out.view(np.float64)
    chunks = 64
    seqs = np.random.SeedSequence(seed).spawn(chunks)
    step = (2 * N) // chunks

    def fill(i):
        part = view[i * step:(i + 1) * step]
        np.random.default_rng(seqs[i]).standard_normal(out=part)
        return float(np.dot(part, part))

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        total = sum(ex.map(fill, range(chunks)))
    out *= 1.0 / np.sqrt(total)
    return out


def test_gate_mix_30_qubits_amplitudes(dfs, oracle):
    if host_ram_bytes() < (48 << 30):
        pytest.skip("the 30-qubit oracle needs about 48 GiB of host memory")
    n = N_QUBITS
    gates = circuits.gate_mix(n, 200, CIRCUIT_SEED)
    amps = seeded_state(n, 11)
    states = {}
    for prec in ("c128", "c128_native"):
        s = dfs.StateVector(n, precision=prec)
        s.setAmps(amps)
        states[prec] = s
    t0 = time.perf_counter()
    for s in states.values():
        circuits.apply(dfs, s, gates)
    dfs.comm_synch()
    t_gpu = time.perf_counter() - t0
    t0 = time.perf_counter()
    circuits.apply_to(oracle, amps, gates)
    t_oracle = time.perf_counter() - t0
    big = float(np.max(np.abs(amps)))
    buf = np.empty(CHUNK, dtype=np.complex128)
    for prec, s in states.items():
        worst = 0.0
        for start in range(0, 1 << n, CHUNK):
            dfs._lib.call("dfs_state_get_amps", s.handle, buf.ctypes.data_as(C.POINTER(C.c_double)), start, CHUNK)
            worst = max(worst, float(np.max(np.abs(buf - amps[start:start + CHUNK]))))
        err = worst / big
        print(f"{prec}: max |engine - oracle| / max |oracle| = {err:.3e} "
              f"(engine {t_gpu:.1f} s for both forms, oracle {t_oracle:.1f} s)")
        assert err <= 1e-12, (prec, err)
        s.free()

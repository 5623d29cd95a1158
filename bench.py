"""Benchmarks of the GB300 statevector / density-matrix engine.

Default workload (the headline): fused-gate application on a 30-qubit
quantum-volume-style circuit — 30 layers, each a seeded random pairing of
the qubits with one Haar-random SU(4) per pair (450 two-qubit unitaries) —
fused by Aer's Fusion pass (max 5 qubits; it yields 218 fused ops), with the
2^30-amplitude complex128 state (17 GB) resident in HBM.  One step applies
the whole fused circuit once.  The same line carries the complex64 run of the
same circuit under ``variants``.

  value    fused-gate GB/s = fused ops x (2 x 2^n x bytes/amp) / step time:
           the algorithmic bytes of one read+write pass per fused op
  e2e      the same metric through the public API (AerSimulator-shaped
           compile+run through the C ABI) with |psi0> uploaded from pinned
           host memory and the 8-qubit marginal read back, every step
  roofline the dominant kernel (the fused 4-qubit ops over the state): its
           algorithmic bytes per launch / its mean launch time over every
           4-qubit op of one pass (CUDA events on the engine's stream),
           against the measured HBM copy bandwidth;
           traffic = DRAM bytes per launch from an ncu capture of the same
           kernel on a 26-qubit state, scaled by 16 (traffic grows with the
           state)
  parity   after the timed region: |0> through the fused circuit and back
           through every op's inverse at the full size (max amplitude error,
           reduced on the GPU), and the same circuit family at 26 qubits
           against the complex128 oracle applying every unfused SU(4)
  cpu_baseline  the oracle (C restatement of Aer's QubitVector + OpenMP) on
           the host cores, a bounded sample of the same fused ops applied to
           the same 2^30-amplitude complex128 state in host memory
  variants the complex64 run of the same circuit; the adjoint gradient of the
           26-qubit, 624-parameter ansatz (complex128 and complex64) against
           parameter shift on the same GPU; the 14-qubit noisy density matrix;
           100,000 shots on the 30-qubit state; the EstimatorV2 job and the
           2,048-instance batch (complex64 and complex128), each as its own
           workload below

Other workloads (--workload): ``adjoint`` (26-qubit hardware-efficient
ansatz, 624 parameters, 200 Pauli terms: adjoint gradient vs parameter
shift), ``dm`` (14-qubit noisy density matrix, depolarizing + amplitude
damping superoperators, 50 Pauli expectation values), ``sample``
(probabilities and 100,000 shots on the 30-qubit state), ``batch`` (2,048
uneven instances of 12-22 qubits with gradients and 4,096 shots each in one
graph-captured persistent launch, next to one instance per launch),
``estimator`` (EstimatorV2 job: a parameterised 20-qubit ansatz with 1,024
parameter sets run on one stack of states, 50 observables), ``shots``
(a 16-qubit circuit with mid-circuit measurements, conditioned gates and
resets: 4,096 shots, each running the circuit, stacked as states),
``noisy`` (a 16-qubit circuit of 188 noisy gates on the statevector method,
each error a Kraus channel drawn per shot: 4,096 shots stacked as states),
``dense5`` (5-qubit Haar gates on a dense 30-qubit state: the 5-qubit
tensor-core kernels), ``tune`` (a 28-qubit unfused ansatz through
AerSimulator.run with the default schedule and with autotune=True).

``--impl reference`` times the reference's CPU algorithm on the same
workload (the oracle port: the reference's own build exists only where its
sources do, not on the GPU host), all host threads, bounded per step: the
same 30-qubit complex128 state in host memory and the same fused ops, read
from the file build() writes, so that the arm maps no engine library.
States of 2^26 amplitudes and more exceed L2 (129 MB), so no flush is needed.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__ as entry  # noqa: E402

MEASURED = ROOT / "MEASURED_PEAKS.json"


def haar_su4(rng):
    z = (rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    q = q * (np.diag(r) / np.abs(np.diag(r)))
    return q / np.linalg.det(q) ** 0.25


def qv_circuit(P, n, layers, seed):
    rng = np.random.default_rng(seed)
    qc = P.QuantumCircuit(n)
    for _ in range(layers):
        perm = rng.permutation(n)
        for a, b in zip(perm[0::2], perm[1::2]):
            qc.unitary(haar_su4(rng), [int(a), int(b)])
    return qc


def hbm_peak():
    if MEASURED.exists():
        d = json.loads(MEASURED.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        q = "clocks.sm,clocks.max.sm," + ",".join("clocks_event_reasons." + f for f in self.FIELDS)

        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-i", "0"],
                                         capture_output=True, text=True, timeout=5).stdout.strip()
                    if out:
                        self.samples.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)

        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()
        return self

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=5)
        num = lambda v: v.replace(".", "", 1).isdigit()
        sm = [float(s[0]) for s in self.samples if s and num(s[0])]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and num(s[1])]
        reasons = sorted({f for s in self.samples for i, f in enumerate(self.FIELDS)
                          if len(s) > 2 + i and s[2 + i].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


class Timer:
    """CUDA events recorded on the engine's own stream."""

    def __init__(self, torch, stream_ptr):
        self.torch = torch
        self.stream = torch.cuda.ExternalStream(stream_ptr)

    def __enter__(self):
        self.e0 = self.torch.cuda.Event(enable_timing=True)
        self.e1 = self.torch.cuda.Event(enable_timing=True)
        self.e0.record(self.stream)
        return self

    def __exit__(self, *a):
        self.e1.record(self.stream)
        self.e1.synchronize()
        self.ms = self.e0.elapsed_time(self.e1)


def oracle_sample(fused_ops, n, budget_s=12.0, max_ops=None):
    """The oracle (C restatement of Aer's QubitVector::apply_matrix, OpenMP on
    every host core) applying the workload's fused ops, in order, to a
    2^n-amplitude complex128 state on the host: a bounded sample (one untimed
    op first touches the state's pages).  Returns (GB/s, ops, seconds, threads)."""
    from oracle import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads, 14)
    o = O.OracleQV(n)
    o.apply_matrix(*fused_ops[0])
    t0 = time.perf_counter()
    done = 0
    while time.perf_counter() - t0 < budget_s and (max_ops is None or done < max_ops):
        q, m = fused_ops[(1 + done) % len(fused_ops)]
        o.apply_matrix(q, m)
        done += 1
    dt = time.perf_counter() - t0
    del o
    return done * 2 * (1 << n) * 16 / dt / 1e9, done, dt, threads


def cpu_baseline(fused_ops, n, budget_s=12.0):
    gbs, done, dt, threads = oracle_sample(fused_ops, n, budget_s)
    return {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"{done} fused ops of the workload on the {n}-qubit complex128 state "
                      f"({(1 << n) * 16 / 1e9:.2f} GB in host memory), {dt:.1f} s wall, OpenMP {threads} threads"}


def fused_ops_of(P, args):
    qc = qv_circuit(P, args.qubits, args.layers, args.seed)
    segs, _, _, meta = P.AerSimulator(precision=args.precision).compile(qc)
    nc = segs[0][1]
    return qc, nc, [(q, nc.op_matrix(i)) for i, (_, _, q) in enumerate(nc.ops())]


def qv_config(args, nops):
    """The workload description both arms print (identical by construction)."""
    return {"workload": f"QV {args.qubits}q x {args.layers} layers (Haar SU(4) per pair), Aer fusion max 5",
            "qubits": args.qubits, "layers": args.layers, "seed": args.seed, "fused_ops": nops,
            "l2": "state larger than L2, no flush" if (16 << args.qubits) > 129e6 else "state fits L2, no flush"}


def ops_file(qubits, layers, seed):
    return ROOT / "_build" / "bench_ops" / f"qv_{qubits}q_{layers}l_seed{seed}_fused.npz"


def export_fused_ops(P=None, qubits=30, layers=30, seed=2024):
    """Writes the fused op list of the QV workload (Aer's Fusion, max 5 qubits)
    to a numpy file, so that the reference arm reads its input with numpy
    alone and never maps the engine's library."""
    P = P or entry.load_package()
    args = argparse.Namespace(qubits=qubits, layers=layers, seed=seed, precision="double")
    _, _, fused = fused_ops_of(P, args)
    path = ops_file(qubits, layers, seed)
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez(str(path) + ".tmp.npz", k=np.array([len(q) for q, _ in fused], dtype=np.int32),
             qubits=np.concatenate([np.asarray(q, dtype=np.uint64) for q, _ in fused]),
             mats=np.concatenate([np.asarray(m, dtype=np.complex128).reshape(-1) for _, m in fused]))
    os.replace(str(path) + ".tmp.npz", path)
    return path


def load_fused_ops(path):
    d = np.load(path)
    out, qo, mo = [], 0, 0
    for k in d["k"]:
        k = int(k)
        dim = 1 << k
        # stored as the engine's column-major vector; the 2-D matrix is U itself
        out.append(([int(x) for x in d["qubits"][qo:qo + k]],
                     d["mats"][mo:mo + dim * dim].reshape(dim, dim, order="F")))
        qo += k
        mo += dim * dim
    return out


def run_reference_arm(args):
    """The reference's CPU algorithm (the oracle port of QubitVector::apply_matrix,
    every host thread) on the same 30-qubit state and the same fused ops, read
    from the file build() writes; each step a bounded sample of the circuit's
    ops (--ref-ops-per-step, continuing through the list)."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    path = ops_file(args.qubits, args.layers, args.seed)
    if not path.exists():
        # the fused list is written by build(); make it in a child process so
        # this process maps no engine library
        subprocess.run([sys.executable, "-c", "import bench; bench.export_fused_ops("
                        f"qubits={args.qubits}, layers={args.layers}, seed={args.seed})"], cwd=ROOT, check=True)
    fused = load_fused_ops(path)
    from oracle import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads, 14)
    n = args.qubits
    o = O.OracleQV(n)
    pos = [0]

    def step():
        for _ in range(args.ref_ops_per_step):
            q, m = fused[pos[0] % len(fused)]
            o.apply_matrix(q, m)
            pos[0] += 1

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    nops = args.steps * args.ref_ops_per_step
    v = round(nops * 2 * (1 << n) * 16 / dt / 1e9, 3)
    print(json.dumps({
        "metric": "fused-gate GB/s", "value": v, "unit": "GB/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": qv_config(args, len(fused)),
        "cpu_baseline": {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{args.ref_ops_per_step} fused ops per step of the workload's {len(fused)}, "
                                   f"applied in circuit order to the {n}-qubit complex128 state "
                                   f"({(1 << n) * 16 / 1e9:.1f} GB in host memory), {nops} ops timed in "
                                   f"{dt:.1f} s, OpenMP {threads} threads"},
        "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


class _DeviceArray:
    """A device buffer the engine owns, described to torch without a copy."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


def roundtrip_err(torch, P, st, nc, fused):
    """Full-size check: |0> through the fused circuit and then through the
    inverse of every fused op (U^dagger, in reverse order) must return to |0>;
    max |amplitude - delta_0| over the 2^n amplitudes, reduced on the GPU."""
    L = P.lib()
    st.initialize()
    A_check(L, L.gbqv_execute(st.handle, nc.handle), st)
    for q, m in reversed(fused):
        dim = 1 << len(q)
        u = np.asarray(m).reshape(dim, dim, order="F") if np.ndim(m) == 1 else np.asarray(m)
        st.apply_matrix(q, u.conj().T)
    st.synchronize()
    typestr = "<c16" if st.precision == "double" else "<c8"
    t = torch.as_tensor(_DeviceArray(st.device_pointer(), 1 << st.num_qubits(), typestr), device="cuda")
    err = max(abs(complex(t[0].item()) - 1.0), float(t[1:].abs().max().item()))
    del t
    torch.cuda.empty_cache()
    return err


_ORACLE_STATES = {}


def err_vs_oracle(P, args, n):
    """The QV family at n qubits (same layers and seed) through the engine
    (fused, the headline's kernels), against the oracle applying every unfused
    SU(4) in complex128: max |amplitude difference|."""
    from oracle import oracle as O

    qc = qv_circuit(P, n, args.layers, args.seed)
    key = (n, args.layers, args.seed)
    if key not in _ORACLE_STATES:
        O.build()
        O.set_threads(os.cpu_count() or 1, 14)
        o = O.OracleQV(n)
        for ins in qc.data:
            o.apply_matrix(ins.qubits, ins.data)
        _ORACLE_STATES[key] = o.data.copy()
        del o
    segs, _, _, _ = P.AerSimulator(precision=args.precision).compile(qc)
    L = P.lib()
    st = P.QubitVector(n, args.precision)
    st.initialize()
    A_check(L, L.gbqv_execute(st.handle, segs[0][1].handle), st)
    sv = st.copy_to_vector()
    st.close()
    return float(np.max(np.abs(sv - _ORACLE_STATES[key])))


# DRAM bytes (read + write) per launch of the dominant kernel, from
# `ncu --set full` captures on a 26-qubit state (profiles/k_dense_tc4_c128_26q.md,
# profiles/k_dense_tc4_c64_26q.md), scaled to 2^qubits amplitudes.
NCU_TRAFFIC_26Q = {("c128", 4): 2.0923e9, ("c64", 4): 1.0134e9}


def bench_qv(args, torch, P):
    L = P.lib()
    qc, nc, fused = fused_ops_of(P, args)
    nops = len(fused)
    amp_bytes = 16 if args.precision == "double" else 8
    pass_bytes = 2 * (1 << args.qubits) * amp_bytes
    st = P.QubitVector(args.qubits, args.precision)
    if args.no_blocking:
        A_check(L, L.gbqv_set_blocking(st.handle, 0), st)
    timer = lambda: Timer(torch, st.stream())

    def step():
        A_check(L, L.gbqv_execute(st.handle, nc.handle), st)

    st.initialize()
    # at least two warm-up steps: runs that recur are compiled for their op
    # sequence on their second execution, which must not land in the timing
    for _ in range(max(args.warmup, 2)):
        step()
    st.synchronize()
    clocks = ClockSampler().start()
    n0 = L.gbqv_launch_count()
    with timer() as t:
        for _ in range(args.steps):
            step()
    launches = (L.gbqv_launch_count() - n0) // max(args.steps, 1)
    clk = clocks.stop()
    t_step = t.ms / 1e3 / args.steps
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        tt = torch.tensor([t_step], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_step = float(tt.item())
    value = nops * pass_bytes / t_step / 1e9 * world
    # dominant kernel: every fused 4-qubit op of one more pass over the
    # circuit, each bracketed by CUDA events on the engine's stream; achieved
    # = algorithmic bytes per launch / mean launch time over those ops
    stream = torch.cuda.ExternalStream(st.stream())
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(nops + 1)]
    st.synchronize()
    evs[0].record(stream)
    for i, (q, m) in enumerate(fused):
        st.apply_matrix(q, m)
        evs[i + 1].record(stream)
    evs[-1].synchronize()
    per_op = [evs[i].elapsed_time(evs[i + 1]) for i in range(nops)]
    k4 = [t for t, (q, _) in zip(per_op, fused) if len(q) == 4] or per_op
    ms_launch = float(np.mean(k4))
    peak, peak_kind = hbm_peak()
    achieved = pass_bytes / (ms_launch / 1e3) / 1e9
    q4 = next((q for q, _ in fused if len(q) == 4), fused[0][0])
    dtype = "c128" if args.precision == "double" else "c64"
    traffic = NCU_TRAFFIC_26Q.get((dtype, len(q4)))
    kname = {"c128": "k_dense_tc4 (tcgen05, exact digit slices)",
             "c64": "k_dense_tc4_c64 (tcgen05, 3xTF32 split precision)"}[dtype]
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4),
            "traffic": round(traffic * 2.0 ** (args.qubits - 26)) if traffic else None,
            "kernel": f"{kname}: mean over the {len(k4)} dense {len(q4)}-qubit ops of a pass, "
                      f"{ms_launch:.3f} ms/launch (min {min(k4):.3f}, max {max(k4):.3f}), "
                      f"{pass_bytes / 1e9:.2f} GB algorithmic per launch", "peak_kind": peak_kind}
    # e2e: public API with host buffers
    e2e = None
    if args.qubits <= 31:
        # |psi0> in pinned (page-locked) host memory, allocated before the timed region
        psi0_t = torch.zeros(1 << args.qubits, dtype=torch.complex128, pin_memory=True)
        psi0 = psi0_t.numpy()
        psi0[0] = 1.0
        sim = P.AerSimulator(precision=args.precision, blocking_enable=not args.no_blocking)

        parts = np.zeros(4)

        def e2e_step():
            t = [time.perf_counter()]
            segs, _, _, _ = sim.compile(qc)        # Fusion pass on the host
            t.append(time.perf_counter())
            st.initialize_from_vector(psi0)        # H2D (returns when the copy is done)
            t.append(time.perf_counter())
            A_check(L, L.gbqv_execute(st.handle, segs[0][1].handle), st)
            st.synchronize()
            t.append(time.perf_counter())
            st.probabilities(list(range(8)))       # D2H of a marginal
            t.append(time.perf_counter())
            parts[:] += np.diff(t)

        e2e_step()                                 # warm-up: staging buffers, first use of psi0's pages
        st.synchronize()
        parts[:] = 0
        t1 = time.perf_counter()
        for _ in range(max(1, args.steps)):
            e2e_step()
        st.synchronize()
        te = (time.perf_counter() - t1) / max(1, args.steps)
        parts /= max(1, args.steps)
        e2e = {"value": round(nops * pass_bytes / te / 1e9, 3), "unit": "GB/s", "ms_per_step": round(te * 1e3, 2),
               "h2d_bytes_per_step": int(psi0.nbytes), "d2h_bytes_per_step": 8 * 256,
               "breakdown_ms": {k: round(float(v) * 1e3, 2) for k, v in
                                zip(("fusion", "upload", "execute", "readback"), parts)}}
        del psi0, psi0_t
    # parity at the full size (inverse round trip, on the device) and against
    # the oracle at the largest size it finishes in seconds
    checks = None
    if not args.no_checks:
        checks = {"roundtrip_max_abs_err": roundtrip_err(torch, P, st, nc, fused),
                  "roundtrip": f"|0> through the {nops} fused ops and their inverses at {args.qubits} qubits, "
                               "max |amp - delta_0| over every amplitude"}
    st.close()
    if not args.no_checks:
        n_or = min(args.qubits, args.oracle_qubits)
        checks["err_vs_oracle"] = err_vs_oracle(P, args, n_or)
        checks["oracle"] = (f"QV {n_or}q x {args.layers} layers (seed {args.seed}) through the engine, "
                            "max |amp - oracle| against the complex128 oracle applying every unfused SU(4)")
    base = None
    if int(os.environ.get("RANK", "0")) == 0 and not args.no_cpu_baseline:
        base = cpu_baseline(fused, args.qubits)
    variants = None
    if args.precision == "double" and not args.no_variants:
        v64 = argparse.Namespace(**{**vars(args), "precision": "single", "no_cpu_baseline": True,
                                    "no_variants": True, "steps": max(2, args.steps), "warmup": 3})
        r = bench_qv(v64, torch, P)
        variants = {"c64": {k: r[k] for k in ("value", "unit", "ms_per_step", "gpu_launches", "roofline", "e2e",
                                              "parity")}}
        for prec in ("double", "single"):
            va = argparse.Namespace(**{**vars(args), "precision": prec, "qubits": 26, "steps": 2, "warmup": 1})
            r = bench_adjoint(va, torch, P)
            variants["adjoint_" + ("c128" if prec == "double" else "c64")] = {
                k: r[k] for k in ("value", "unit", "adjoint_s", "param_shift_s_extrapolated", "param_shift_measured",
                                  "rel_err_vs_param_shift", "energy_err_vs_oracle", "config")}
        vd = argparse.Namespace(**{**vars(args), "precision": "double", "steps": 3, "warmup": 1})
        r = bench_dm(vd, torch, P)
        variants["dm14_c128"] = {k: r[k] for k in ("value", "unit", "ms_per_step", "fused_ops",
                                                   "expval_50_terms_ms", "config")}
        # the other workloads (sampling, parameter binding, batched instances),
        # so that every headline number has a record in this line
        vs = argparse.Namespace(**{**vars(args), "no_checks": True})
        r = bench_sample(vs, torch, P)
        variants["sample_30q_c128"] = {k: r[k] for k in ("value", "unit", "sample_100k_ms", "probabilities_all_ms",
                                                         "config")}
        ve = argparse.Namespace(**{**vars(args), "precision": "single", "steps": 3, "warmup": 3,
                                   "per_binding_sample": 1, "no_cpu_baseline": True})
        r = bench_estimator(ve, torch, P)
        variants["estimator_c64"] = {k: r[k] for k in ("value", "unit", "ms_per_step", "execute_bound_ms",
                                                       "expval_50_terms_ms", "e2e", "config")}
        vb = argparse.Namespace(**{**vars(args), "precision": "single", "steps": 2, "warmup": 1,
                                   "no_cpu_baseline": True})
        r = bench_batch(vb, torch, P)
        variants["batch_c64"] = {k: r[k] for k in ("value", "unit", "launch_ms", "latency_ms_p50", "latency_ms_p99",
                                                   "speedup_vs_per_launch", "config")}
        # the same two at complex128 (float-pair arithmetic on the FP32 pipe)
        ve2 = argparse.Namespace(**{**vars(ve), "precision": "double", "steps": 1, "warmup": 2})
        r = bench_estimator(ve2, torch, P)
        variants["estimator_c128"] = {k: r[k] for k in ("value", "unit", "ms_per_step", "execute_bound_ms",
                                                        "expval_50_terms_ms", "e2e", "config")}
        vb2 = argparse.Namespace(**{**vars(vb), "precision": "double", "steps": 1})
        r = bench_batch(vb2, torch, P)
        variants["batch_c128"] = {k: r[k] for k in ("value", "unit", "launch_ms", "latency_ms_p50", "latency_ms_p99",
                                                    "speedup_vs_per_launch", "config")}
    return {"metric": "fused-gate GB/s", "value": round(value, 3), "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128" if args.precision == "double" else "c64", "data": "synthetic",
            "config": qv_config(args, nops), "engine": {"blocking": not args.no_blocking},
            "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": base, "e2e": e2e, "clocks": clk,
            "parity": checks, "variants": variants}


def bench_dense5(args, torch, P):
    """5-qubit dense gates: per layer a seeded permutation of the qubits into
    groups of five, a Haar-random 32 x 32 unitary on each (the width Aer's
    Fusion reaches with max_fusion_qubits = 5), applied one op per launch to
    the 2^qubits state in HBM, made dense first (untimed Hadamards)."""
    rng = np.random.default_rng(args.seed)
    n = args.qubits
    ops = []
    for _ in range(args.dense5_layers):
        perm = rng.permutation(n)
        for g in range(n // 5):
            z = rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32))
            q, r = np.linalg.qr(z)
            ops.append(([int(x) for x in perm[5 * g:5 * g + 5]], q * (np.diag(r) / np.abs(np.diag(r)))))
    st = P.QubitVector(n, args.precision)
    st.initialize()
    stream = torch.cuda.ExternalStream(st.stream())
    # a dense state first (Hadamard on every qubit), so that no group of the
    # timed gates is all zero (the tensor kernels skip the stores of those)
    h = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    for q in range(n):
        st.apply_matrix([q], h)
    for q, m in ops[:args.warmup]:
        st.apply_matrix(q, m)
    st.synchronize()
    L = P.lib()
    n0 = L.gbqv_launch_count()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(len(ops) + 1)]
    evs[0].record(stream)
    for i, (q, m) in enumerate(ops):
        st.apply_matrix(q, m)
        evs[i + 1].record(stream)
    evs[-1].synchronize()
    launches = L.gbqv_launch_count() - n0
    per = [evs[i].elapsed_time(evs[i + 1]) for i in range(len(ops))]
    norm = st.norm()
    st.close()
    amp = 16 if args.precision == "double" else 8
    pass_bytes = 2 * (1 << n) * amp
    ms = float(np.mean(per))
    peak, kind = hbm_peak()
    flops = 8 * 32 * (1 << n)
    return {"metric": "5-qubit dense gate GB/s", "value": round(pass_bytes / ms / 1e6, 1), "unit": "GB/s",
            "higher_is_better": True, "n_gpus": 1, "dtype": "c128" if args.precision == "double" else "c64",
            "data": "synthetic", "ms_per_gate": round(ms, 4), "min_ms": round(min(per), 4),
            "gates": len(ops), "gpu_launches": int(launches), "norm_after": norm,
            "roofline": {"bound": "hbm", "achieved": round(pass_bytes / ms / 1e6, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(pass_bytes / ms / 1e6 / peak, 4), "peak_kind": kind,
                         "flops_per_gate": flops, "tflops": round(flops / ms / 1e9, 1)},
            "config": {"workload": f"{n}q, {args.dense5_layers} layers of {n // 5} Haar SU(32) on disjoint 5-qubit groups",
                       "qubits": n}}


def A_check(L, rc, st):
    if rc != 0:
        raise RuntimeError(L.gbqv_last_error(st.handle).decode())


_ORACLE_ENERGY = {}


def oracle_energy(ans, theta, ham, key):
    """<H> of the ansatz state from the complex128 oracle (every gate applied
    one by one, then each Pauli term's expectation value)."""
    if key not in _ORACLE_ENERGY:
        from oracle import oracle as O

        O.build()
        O.set_threads(os.cpu_count() or 1, 14)
        o = O.OracleQV(ans.num_qubits)
        axis = {"rx": 0, "ry": 1, "rz": 2}
        for ins in ans.instructions(theta):
            if ins.name in axis:
                o.apply_rotation(ins.qubits, axis[ins.name], ins.params[0])
            elif ins.name == "cx":
                o.apply_mcx(ins.qubits)
            else:
                raise ValueError(f"oracle_energy: gate {ins.name} is not in the ansatz family")
        _ORACLE_ENERGY[key] = sum(c * o.expval_pauli(q, lab) for (q, lab), c in zip(ham.terms, ham.coeffs))
    return _ORACLE_ENERGY[key]


def bench_adjoint(args, torch, P):
    """26 qubits, 12 layers of RY/RZ on every qubit + a CX ladder (624
    parameters), 200 Pauli terms of weight 1-4 with N(0,1) coefficients."""
    adj = P.adjoint
    rng = np.random.default_rng(args.seed)
    n, layers = args.qubits if args.qubits != 30 else 26, 12
    ans = adj.hardware_efficient_ansatz(n, layers)
    ham = adj.random_hamiltonian(n, 200, rng)
    theta = rng.uniform(-np.pi, np.pi, ans.num_params)
    eng = adj.Engine(n, args.precision)
    # at least two warm-up calls: runs that recur are compiled for their op
    # sequence on their second execution, which must not land in the timing
    for _ in range(max(args.warmup, 2)):
        eng.energy_and_grad(ans, theta, ham)
    clocks = ClockSampler().start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e, g = eng.energy_and_grad(ans, theta, ham)
    t_adj = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    # parameter shift on a subset, same engine; extrapolated to all parameters
    idx = [int(i) for i in rng.choice(ans.num_params, size=args.shift_params, replace=False)]
    for _ in range(2):  # the same for parameter shift's forward passes
        eng.energy(ans, theta, ham)
    t1 = time.perf_counter()
    ps = eng.param_shift_grad(ans, theta, ham, idx)
    t_ps_sub = time.perf_counter() - t1
    t_ps = t_ps_sub / len(idx) * ans.num_params
    ps_v = np.array([ps[i] for i in idx])
    rel = float(np.linalg.norm(g[idx] - ps_v) / np.linalg.norm(ps_v))
    eng.close()
    e_err = None
    if not args.no_checks:
        e_err = abs(e - oracle_energy(ans, theta, ham, (n, args.seed)))
    return {"metric": "adjoint-grad time vs param-shift", "value": round(t_ps / t_adj, 2), "unit": "x faster",
            "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "dtype": "c128" if args.precision == "double" else "c64", "data": "synthetic",
            "adjoint_s": round(t_adj, 4), "param_shift_s_extrapolated": round(t_ps, 2),
            "param_shift_measured": f"{len(idx)} params x 2 evaluations in {t_ps_sub:.2f} s",
            "rel_err_vs_param_shift": rel, "energy": e, "energy_err_vs_oracle": e_err,
            "config": {"workload": f"HEA {n}q x {layers} layers, {ans.num_params} params, 200 Pauli terms",
                       "qubits": n}, "clocks": clk}


def bench_dm(args, torch, P):
    """14-qubit density matrix: 40 layers of U3 on every qubit + CX on a seeded
    pairing; after every gate depolarizing p=1e-3 and amplitude damping
    gamma=2e-3 (4x4 / 16x16 superoperators); 50 random Pauli expvals."""
    rng = np.random.default_rng(args.seed)
    n, layers = 14, args.dm_layers
    e1 = P.depolarizing_error(1e-3, 1).compose(P.amplitude_damping_error(2e-3))
    nm = P.NoiseModel()
    nm.add_all_qubit_quantum_error(e1, ["u3"])
    nm.add_all_qubit_quantum_error(e1.tensor(e1), ["cx"])
    qc = P.QuantumCircuit(n)
    for _ in range(layers):
        for q in range(n):
            qc.u3(*rng.uniform(0, 2 * np.pi, 3), q)
        perm = rng.permutation(n)
        for a, b in zip(perm[0::2], perm[1::2]):
            qc.cx(int(a), int(b))
    terms = []
    for _ in range(50):
        k = int(rng.integers(1, 5))
        q = [int(x) for x in rng.choice(n, k, replace=False)]
        terms.append((float(rng.normal()), "".join(rng.choice(list("IXYZ"), k)), q))
    qc.save_expectation_value(terms)
    sim = P.AerSimulator(method="density_matrix", noise_model=nm, precision=args.precision)
    segs, _, _, meta = sim.compile(qc)
    nops = segs[0][1].num_ops()
    L = P.lib()
    st = P.DensityMatrix(n, args.precision)
    for _ in range(max(args.warmup, 2)):
        st.initialize()
        A_check(L, L.gbqv_execute(st.handle, segs[0][1].handle), st)
    st.synchronize()
    clocks = ClockSampler().start()
    with Timer(torch, st.stream()) as t:
        for _ in range(args.steps):
            st.initialize()
            A_check(L, L.gbqv_execute(st.handle, segs[0][1].handle), st)
    clk = clocks.stop()
    t_step = t.ms / 1e3 / args.steps
    t2 = time.perf_counter()
    vals, total = st.expval_pauli_many([(q, lab) for _, lab, q in terms], [c for c, _, _ in terms])
    t_exp = time.perf_counter() - t2
    st.close()
    amp = 16 if args.precision == "double" else 8
    gbs = nops * 2 * (1 << (2 * n)) * amp / t_step / 1e9
    return {"metric": "fused superop GB/s (density matrix)", "value": round(gbs, 2), "unit": "GB/s",
            "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t_step * 1e3, 2), "dtype": "c128" if args.precision == "double" else "c64",
            "data": "synthetic", "fused_ops": nops, "fusion": meta["fusion"],
            "expval_50_terms_ms": round(t_exp * 1e3, 2), "expval_total": total,
            "config": {"workload": f"DM {n}q x {layers} layers + depolarizing/amp-damping superops", "qubits": n},
            "clocks": clk}


def bench_sample(args, torch, P):
    """probabilities() of all qubits and 100,000 shots from seeded uniforms."""
    L = P.lib()
    qc, nc, fused = fused_ops_of(P, args)
    st = P.QubitVector(args.qubits, args.precision)
    st.initialize()
    A_check(L, L.gbqv_execute(st.handle, nc.handle), st)
    rnds = P.uniforms(args.seed, 100_000)
    st.sample_measure(rnds[:1000])
    t0 = time.perf_counter()
    s = st.sample_measure(rnds)
    t_s = time.perf_counter() - t0
    t1 = time.perf_counter()
    pm = st.probabilities(list(range(10)))
    t_p = time.perf_counter() - t1
    t2 = time.perf_counter()
    pall = st.probabilities()
    t_all = time.perf_counter() - t2
    del pall
    # the first shots against the oracle (the reference's walk, all host cores) on the same state
    check = None
    if not args.no_checks:
        from oracle import oracle as O

        O.build()
        O.set_threads(os.cpu_count() or 1, 14)
        o = O.OracleQV(args.qubits, st.copy_to_vector())
        m = min(args.sample_check, rnds.size)
        want = o.sample_measure(rnds[:m])
        check = {"shots_compared": int(m), "identical": bool(np.array_equal(want, s[:m]))}
        del o
    st.close()
    return {"metric": "shots/s", "value": round(1e5 / t_s, 1), "unit": "shots/s", "higher_is_better": True,
            "n_gpus": 1, "dtype": "c128" if args.precision == "double" else "c64", "data": "synthetic",
            "sample_100k_ms": round(t_s * 1e3, 2), "marginal_10q_ms": round(t_p * 1e3, 2),
            "probabilities_all_ms": round(t_all * 1e3, 2), "vs_oracle": check,
            "config": {"workload": f"QV {args.qubits}q state, 100k shots", "qubits": args.qubits}}


def bench_batch(args, torch, P):
    """2,048 instances: n ~ U{12..22}, depth ~ U{4..16} layers of the RY/RZ +
    CX-ladder ansatz, own theta, 20-60-term Pauli H, 4,096 shots each; <H>,
    gradient and shots per instance in one graph-captured persistent launch,
    next to one instance per launch (the per-instance engine) on a sample."""
    B, adj = P.batched, P.adjoint
    insts = B.config5_instances(args.instances, seed=args.seed, qmin=args.batch_qmin, qmax=args.batch_qmax,
                                dmin=args.batch_dmin, dmax=args.batch_dmax)
    tuned = None
    if args.autotune:  # team split picked by timing the whole batch under each candidate (untimed here)
        T = P.autotune
        tuned = T.tune_batch(insts, args.precision, True, T.Autotuner(warmup=1, repeats=1))
    b = B.Batch(args.precision)
    if tuned is not None:
        b.set_teams(*tuned)
    for inst in insts:
        b.add(inst["n"], inst["gates"], inst["theta"], inst["terms"], inst["coeffs"], inst["shots"], inst["seed"])
    for _ in range(max(1, args.warmup)):
        b.run(want_grad=True)          # first call builds, uploads and captures the graph
    clocks = ClockSampler().start()
    times = [b.run(want_grad=True) for _ in range(args.steps)]
    clk = clocks.stop()
    ms = float(np.median(times))
    lat = np.array([b.result(i)[3] for i in range(len(insts))])
    # one instance per launch: the same work through the per-instance engine, on a sample
    rng = np.random.default_rng(args.seed + 1)
    sample = [int(i) for i in rng.choice(len(insts), size=min(args.per_launch_sample, len(insts)), replace=False)]
    kinds = {0: "rx", 1: "ry", 2: "rz", 3: "cx", 4: "cz", 5: "h"}
    t_single = 0.0
    for i in sample:
        inst = insts[i]
        gates = [(kinds[k], [q0, q1] if k in (3, 4) else [q0], p if p >= 0 else None, None)
                 for k, q0, q1, p in inst["gates"]]
        ans = adj.Ansatz(inst["n"], gates)
        ham = adj.Hamiltonian(inst["terms"], inst["coeffs"])
        eng = adj.Engine(inst["n"], args.precision)
        t0 = time.perf_counter()
        e, g = eng.energy_and_grad(ans, inst["theta"], ham)
        eng.energy(ans, inst["theta"], ham)
        eng.qv.sample_measure(P.uniforms(inst["seed"], inst["shots"]))
        t_single += time.perf_counter() - t0
        eng.close()
    est_single = t_single / len(sample) * len(insts)
    b.close()
    return {"metric": "circuits/s (batched uneven, adjoint gradients + shots)", "value": round(len(insts) / (ms / 1e3), 2),
            "unit": "circuits/s", "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "dtype": "c128" if args.precision == "double" else "c64", "data": "synthetic",
            "launch_ms": round(ms, 2), "latency_ms_p50": round(float(np.percentile(lat, 50)), 3),
            "latency_ms_p99": round(float(np.percentile(lat, 99)), 3),
            "one_instance_per_launch_s_estimated": round(est_single, 2),
            "one_instance_per_launch_measured": f"{len(sample)} instances in {t_single:.2f} s",
            "speedup_vs_per_launch": round(est_single / (ms / 1e3), 2),
            "config": {"workload": f"{len(insts)} instances, {args.batch_qmin}-{args.batch_qmax} qubits, depth "
                                   f"{args.batch_dmin}-{args.batch_dmax}, 20-60 Paulis, 4096 shots",
                       "instances": len(insts),
                       "teams": list(tuned) if tuned is not None else "default (64, 0.5)"}, "clocks": clk}


def dynamic_circuit(P, n, rounds, seed):
    """Brickwork Haar SU(4) layers; after each round a measurement, an X
    conditioned on it and a reset; at the end every qubit measured."""
    rng = np.random.default_rng(seed)
    qc = P.QuantumCircuit(n, rounds + n)
    for r in range(rounds):
        for start in (0, 1):
            for q in range(start, n - 1, 2):
                qc.unitary(haar_su4(rng), [q, q + 1])
        qc.measure(r % n, r)
        qc.x((r + 1) % n).c_if(r, 1)
        qc.reset([r % n])
    qc.measure(list(range(n)), list(range(rounds, rounds + n)))
    return qc


def bench_shots(args, torch, P):
    """Circuits that cannot be measure-sampled (mid-circuit measurement,
    conditioned gates, resets): every shot runs the circuit, shots stacked
    as states through AerSimulator.run; next to one shot at a time on one
    state (a sample, registers of <= 10 qubits only)."""
    qc = dynamic_circuit(P, args.shots_qubits, args.shots_rounds, args.seed)
    sim = P.AerSimulator(precision=args.precision)
    for _ in range(max(1, args.warmup)):
        sim.run(qc, shots=min(args.shots, 256), seed_simulator=args.seed)
    clocks = ClockSampler().start()
    times = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        counts = sim.run(qc, shots=args.shots, seed_simulator=args.seed + i).get_counts()
        times.append(time.perf_counter() - t0)
    clk = clocks.stop()
    t = float(np.median(times))
    line = {"metric": "shots/s (mid-circuit measurement, reset, conditions)", "value": round(args.shots / t, 1),
            "unit": "shots/s", "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t * 1e3, 2), "dtype": "c128" if args.precision == "double" else "c64",
            "data": "synthetic", "outcomes": len(counts),
            "config": {"workload": f"{args.shots_qubits}q, {args.shots_rounds} rounds of 2 SU(4) layers + measure, "
                                   f"conditioned X, reset; final measure of every qubit; {args.shots} shots",
                       "qubits": args.shots_qubits, "shots": args.shots}, "clocks": clk}
    if args.shots_qubits <= 10:
        one = P.AerSimulator(precision=args.precision)
        one._conditioned_matrices = lambda items: None   # the one-state loop
        ns = min(args.shots, 256)
        t0 = time.perf_counter()
        ref = one.run(qc, shots=ns, seed_simulator=args.seed).get_counts()
        t1 = time.perf_counter() - t0
        same = sim.run(qc, shots=ns, seed_simulator=args.seed).get_counts() == ref
        line["one_shot_at_a_time_shots_per_s"] = round(ns / t1, 1)
        line["speedup_vs_one_shot_at_a_time"] = round((args.shots / t) / (ns / t1), 1)
        line["same_counts_on_sample"] = same
    return line


def noisy_circuit(P, n, layers, seed):
    """U3 with seeded angles on every qubit and CX on alternate pairs, per
    layer; every qubit measured at the end."""
    rng = np.random.default_rng(seed)
    qc = P.QuantumCircuit(n, n)
    for r in range(layers):
        for q in range(n):
            qc.u3(*rng.uniform(0, 2 * np.pi, 3), q)
        for q in range(r % 2, n - 1, 2):
            qc.cx(q, q + 1)
    qc.measure(list(range(n)), list(range(n)))
    return qc


def noisy_model(P, kind):
    """depol: depolarizing 1e-3 on U3 and 1e-2 on CX (mixtures of Paulis);
    damp: depolarizing 1e-3 then amplitude damping 2e-3 on U3, the tensor
    product of two of those on CX (state-dependent Kraus probabilities)."""
    nm = P.NoiseModel()
    if kind == "depol":
        nm.add_all_qubit_quantum_error(P.depolarizing_error(1e-3, 1), ["u3"])
        nm.add_all_qubit_quantum_error(P.depolarizing_error(1e-2, 2), ["cx"])
    else:
        e1 = P.depolarizing_error(1e-3, 1).compose(P.amplitude_damping_error(2e-3))
        nm.add_all_qubit_quantum_error(e1, ["u3"])
        nm.add_all_qubit_quantum_error(e1.tensor(e1), ["cx"])
    return nm


def bench_noisy(args, torch, P):
    """Noise sampled per shot on the statevector method (the reference's
    Kraus noise method): every noisy gate is a Kraus channel drawn per shot,
    shots stacked as states, through AerSimulator.run; next to one shot at a
    time on one state (a sample of 32 shots)."""
    qc = noisy_circuit(P, args.shots_qubits, args.noisy_layers, args.seed)
    nm = noisy_model(P, args.noise)
    sim = P.AerSimulator(precision=args.precision, noise_model=nm)
    for _ in range(max(1, args.warmup)):
        sim.run(qc, shots=min(args.shots, 256), seed_simulator=args.seed)
    clocks = ClockSampler().start()
    times = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        counts = sim.run(qc, shots=args.shots, seed_simulator=args.seed + i).get_counts()
        times.append(time.perf_counter() - t0)
    clk = clocks.stop()
    t = float(np.median(times))
    one = P.AerSimulator(precision=args.precision, noise_model=nm)
    one._conditioned_matrices = lambda items: None   # the one-state loop
    t0 = time.perf_counter()
    one.run(qc, shots=32, seed_simulator=args.seed)
    t1 = time.perf_counter() - t0
    channels = sum(1 for ins in qc.data if ins.kind == "gate")
    return {"metric": "shots/s (noise sampled per shot, statevector)", "value": round(args.shots / t, 1),
            "unit": "shots/s", "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t * 1e3, 2), "dtype": "c128" if args.precision == "double" else "c64",
            "data": "synthetic", "outcomes": len(counts),
            "config": {"workload": f"{args.shots_qubits}q, {args.noisy_layers} layers of U3 + alternate CX, "
                                   f"{channels} noisy gates ({args.noise}); final measure of every qubit; "
                                   f"{args.shots} shots", "qubits": args.shots_qubits, "shots": args.shots},
            "one_shot_at_a_time_shots_per_s": round(32 / t1, 1),
            "speedup_vs_one_shot_at_a_time": round((args.shots / t) / (32 / t1), 1), "clocks": clk}


def hea_bound_circuit(P, n, layers):
    """RY(theta) and RZ(theta) on every qubit, then a CX ladder, per layer;
    one Parameter per rotation (the adjoint workload's ansatz, parameterised)."""
    qc = P.QuantumCircuit(n)
    params = []
    for layer in range(layers):
        for kind in ("ry", "rz"):
            for q in range(n):
                t = P.Parameter(f"t{len(params):04d}")
                params.append(t)
                qc.append_gate(kind, [q], [t])
        for q in range(n - 1):
            qc.cx(q, q + 1)
    return qc, params


def bench_tune(args, torch, P):
    """Autotuned against default schedule: the HEA circuit (RY, RZ on every
    qubit and a CX ladder per layer, fixed angles) without fusion, so that its
    1-2 qubit gates run as cache-blocked runs, through AerSimulator.run with
    one Z expectation value saved; the default engine schedule against
    AerSimulator(autotune=True), whose first call times the execution forms
    and the run tile (untimed here).  Wall time per run() call, median of
    --steps calls each."""
    n, layers = args.tune_qubits, args.tune_layers
    rng = np.random.default_rng(args.seed)
    qc = P.QuantumCircuit(n)
    for _ in range(layers):
        for kind in ("ry", "rz"):
            for q in range(n):
                qc.append_gate(kind, [q], [float(rng.uniform(-np.pi, np.pi))])
        for q in range(n - 1):
            qc.cx(q, q + 1)
    qc.save_expectation_value([(1.0, "Z", [0])], label="z0")
    sims = {"default": P.AerSimulator(precision=args.precision, fusion_enable=False),
            "tuned": P.AerSimulator(precision=args.precision, fusion_enable=False, autotune=True)}
    out, meta, vals = {}, {}, {}
    for name, sim in sims.items():
        for _ in range(max(args.warmup, 2)):  # the tuned simulator tunes on its first call
            res = sim.run(qc)
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = sim.run(qc)
            ts.append(time.perf_counter() - t0)
        out[name] = float(np.median(ts))
        meta[name] = res.metadata(0).get("autotune")
        vals[name] = float(res.data(0)["z0"])
    dtype = "c128" if args.precision == "double" else "c64"
    return {"metric": "circuit time, autotuned vs default schedule", "value": round(out["tuned"] * 1e3, 2),
            "unit": "ms", "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "dtype": dtype,
            "data": "synthetic", "default_ms": round(out["default"] * 1e3, 2),
            "speedup": round(out["default"] / out["tuned"], 3), "choice": meta["tuned"],
            "max_abs_diff_tuned_vs_default": abs(vals["tuned"] - vals["default"]),
            "config": {"workload": f"HEA {n}q x {layers} layers (RY, RZ, CX ladder), no fusion, <Z_0> saved",
                       "qubits": n, "layers": layers}}


def bench_estimator(args, torch, P):
    """EstimatorV2-shaped job: the parameterised HEA ansatz (n qubits x L
    layers) with B parameter sets and 50 Pauli observables of weight 1-4 on
    all qubits.  value = bindings per second with every binding run on one
    stack of 2^b states (gbqv_execute_bound) and the observables reduced per
    state, inputs resident; e2e = EstimatorV2.run([(circuit, observables,
    values)]) end to end (binding table built and uploaded, evs read back);
    next to it the same bindings one at a time through AerSimulator.run
    (the non-batched path) on a sample, and the oracle on the host cores."""
    n, layers, B = args.est_qubits, args.est_layers, args.est_bindings
    dtype = "c128" if args.precision == "double" else "c64"
    rng = np.random.default_rng(args.seed)
    qc, params = hea_bound_circuit(P, n, layers)
    values = rng.uniform(-np.pi, np.pi, size=(B, len(params)))
    labels = []
    for _ in range(50):
        w = int(rng.integers(1, 5))
        lab = ["I"] * n
        for q in rng.choice(n, w, replace=False):
            lab[n - 1 - int(q)] = str(rng.choice(list("XYZ")))
        labels.append("".join(lab))
    terms = [([int(i) for i in range(n)], lab) for lab in labels]
    L = P.lib()
    nc = P.NativeCircuit(n, qc.data)
    binds = {p: values[:, i] for i, p in enumerate(params)}
    nc.bind(binds, B)
    b = (B - 1).bit_length()
    st = P.QubitVector(n + b, args.precision)
    stream = torch.cuda.ExternalStream(st.stream())

    def step():
        P._capi.check(L.gbqv_execute_bound(st.handle, nc.handle, 0, B), st.handle)
        return st.expval_pauli_segments(n, B, terms)

    for _ in range(max(args.warmup, 2)):
        evs = step()
    st.synchronize()
    clocks = ClockSampler().start()
    n0 = L.gbqv_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        evs = step()
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    launches = (L.gbqv_launch_count() - n0) // max(args.steps, 1)
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    # dominant kernel: the bound cache-blocked runs; one execute_bound timed alone
    ex0, ex1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n1 = L.gbqv_launch_count()
    ex0.record(stream)
    P._capi.check(L.gbqv_execute_bound(st.handle, nc.handle, 0, B), st.handle)
    ex1.record(stream)
    ex1.synchronize()
    runs = L.gbqv_launch_count() - n1 - 1           # minus the initialisation kernel
    t_exec = ex0.elapsed_time(ex1) / 1e3
    ex0.record(stream)
    st.expval_pauli_segments(n, B, terms)
    ex1.record(stream)
    ex1.synchronize()
    t_expval = ex0.elapsed_time(ex1) / 1e3
    amp_bytes = 16 if args.precision == "double" else 8
    stack_bytes = (1 << (n + b)) * amp_bytes
    valid_bytes = B * (1 << n) * amp_bytes
    achieved = 2 * valid_bytes * runs / t_exec / 1e9
    peak, peak_kind = hbm_peak()
    # arithmetic: RY then RZ on a qubit run as one 2x2 per binding (8 complex-FMA
    # flops per amplitude and qubit-layer as 8 real FMAs = 16 flops); CX moves data only
    flops = 16.0 * n * layers * B * (1 << n)
    st.close()
    # e2e through the primitive
    est = P.EstimatorV2(options={"backend_options": {"precision": args.precision}})
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = est.run([(qc, labels, values.reshape(B, 1, len(params)))]).result()  # evs: (B, 50)
    t_e2e = (time.perf_counter() - t0) / args.steps
    err = float(np.max(np.abs(res[0].data.evs - evs.T)))
    # one binding at a time on the same GPU (sample)
    sim = P.AerSimulator(precision=args.precision)
    k = min(args.per_binding_sample, B)
    circ1 = qc.copy()
    for lab in labels:
        circ1.save_expectation_value([(1.0, lab, list(range(n)))], label=lab)
    t1 = time.perf_counter()
    for j in range(k):
        sim.run(circ1.assign_parameters(list(values[j])))
    t_one = (time.perf_counter() - t1) / k
    base = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        threads = os.cpu_count() or 1
        O.set_threads(threads, 14)
        t2, done = time.perf_counter(), 0
        while done < 1 or time.perf_counter() - t2 < 10.0:
            o = O.OracleQV(n)
            for ins in qc.data:
                if ins.kind != "gate":
                    continue
                if ins.name == "cx":
                    o.apply_mcx(ins.qubits)
                else:
                    th = float(ins.params[0].bind({p: values[done, i] for i, p in enumerate(params)}))
                    o.apply_rotation(ins.qubits, {"ry": 1, "rz": 2}[ins.name], th)
            for lab in labels:
                o.expval_pauli(list(range(n)), lab)
            done += 1
        dt = time.perf_counter() - t2
        base = {"value": round(done / dt, 3), "unit": "bindings/s", "cores": threads, "kind": "port",
                "sample": f"{done} bindings of the workload (gate by gate + 50 expvals) in {dt:.1f} s, "
                          f"OpenMP {threads} threads"}
    return {"metric": "parameter bindings/s (EstimatorV2, 50 observables)", "value": round(B / t_step, 2),
            "unit": "bindings/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t_step * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": {"workload": f"HEA {n}q x {layers} layers, {len(params)} parameters, {B} bindings, "
                                   f"50 Pauli observables", "qubits": n, "layers": layers, "bindings": B,
                       "stack_qubits": n + b, "l2": "stack larger than L2, no flush"},
            "gpu_launches": int(launches), "execute_bound_ms": round(t_exec * 1e3, 2),
            "expval_50_terms_ms": round(t_expval * 1e3, 2),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": None,
                         "kernel": f"k_run_reg (bound runs): {runs} cache-blocked passes over the {B} states "
                                   f"({valid_bytes / 1e9:.2f} GB) in {t_exec * 1e3:.1f} ms; arithmetic "
                                   f"{flops / t_exec / 1e12:.2f} TFLOP/s"
                                   + (" of the 1.2 TFLOP/s FP64 peak (FP64-bound)" if dtype == "c128" else
                                      " (instruction-issue-bound: per-op register shuffling)"),
                         "peak_kind": peak_kind},
            "e2e": {"value": round(B / t_e2e, 2), "unit": "bindings/s", "ms_per_step": round(t_e2e * 1e3, 2),
                    "h2d_bytes_per_step": int(values.nbytes), "d2h_bytes_per_step": int(B * len(labels) * 8)},
            "one_binding_per_run": {"value": round(1 / t_one, 2), "unit": "bindings/s",
                                    "sample": f"{k} bindings through AerSimulator.run, fused"},
            "max_abs_diff_e2e_vs_device": err, "cpu_baseline": base, "clocks": clk}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="qv",
                    choices=["qv", "adjoint", "dm", "sample", "batch", "estimator", "shots", "noisy", "dense5",
                             "tune"])
    ap.add_argument("--tune-qubits", type=int, default=28)
    ap.add_argument("--tune-layers", type=int, default=8)
    ap.add_argument("--dense5-layers", type=int, default=4)
    ap.add_argument("--shots-qubits", type=int, default=16)
    ap.add_argument("--shots-rounds", type=int, default=8)
    ap.add_argument("--shots", type=int, default=4096)
    ap.add_argument("--noisy-layers", type=int, default=8, help="noisy workload: layers")
    ap.add_argument("--noise", choices=["depol", "damp"], default="damp", help="noisy workload: noise model")
    ap.add_argument("--est-qubits", type=int, default=20)
    ap.add_argument("--est-layers", type=int, default=8)
    ap.add_argument("--est-bindings", type=int, default=1024)
    ap.add_argument("--per-binding-sample", type=int, default=8)
    ap.add_argument("--instances", type=int, default=2048)
    ap.add_argument("--batch-qmin", type=int, default=12)
    ap.add_argument("--batch-qmax", type=int, default=22)
    ap.add_argument("--batch-dmin", type=int, default=4)
    ap.add_argument("--batch-dmax", type=int, default=16)
    ap.add_argument("--per-launch-sample", type=int, default=24)
    ap.add_argument("--precision", default="double", choices=["double", "single"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--layers", type=int, default=30)
    ap.add_argument("--dm-layers", type=int, default=40)
    ap.add_argument("--shift-params", type=int, default=6)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-blocking", action="store_true")
    ap.add_argument("--autotune", action="store_true",
                    help="batch workload: pick the two-CTA team split by timing the candidates first")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the complex64, adjoint and density-matrix runs of the default workload")
    ap.add_argument("--no-checks", action="store_true", help="skip the parity checks of the default workload")
    ap.add_argument("--sample-check", type=int, default=2000,
                    help="sample workload: shots compared with the oracle's walk on the same state")
    ap.add_argument("--oracle-qubits", type=int, default=26,
                    help="state size of the default workload's comparison with the oracle")
    ap.add_argument("--ref-ops-per-step", type=int, default=2,
                    help="reference arm: fused ops of the 30-qubit circuit applied per step")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        torch.distributed.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.init()
    P = entry.load_package()
    P.build()
    fn = {"qv": bench_qv, "adjoint": bench_adjoint, "dm": bench_dm, "sample": bench_sample,
          "batch": bench_batch, "estimator": bench_estimator, "shots": bench_shots, "noisy": bench_noisy,
          "dense5": bench_dense5, "tune": bench_tune}[args.workload]
    line = fn(args, torch, P)
    if int(os.environ.get("RANK", "0")) == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()

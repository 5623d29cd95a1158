"""Headline benchmark: fused-gate application on a 30-qubit quantum-volume
circuit (30 layers of seeded random qubit pairings, one Haar-random SU(4)
per pair = 450 two-qubit unitaries), fused by Aer's Fusion pass
(max_fusion_qubits=5), state resident in HBM.

A step applies the whole fused circuit once to the 2^30-amplitude state.
  value  = fused-gate GB/s = (fused ops x 2 x 2^n x bytes/amp) / step time
           (the algorithmic bytes of one read+write pass per fused op)
  e2e    = the same metric through the public API (AerSimulator-shaped
           run through the C ABI) with the initial state uploaded from
           pinned host memory and the final probabilities of 8 qubits read
           back, every step
  roofline = the dominant kernel's achieved bytes per launch / its mean
           launch time (CUDA events on the engine's stream), against the
           measured HBM copy bandwidth
  cpu_baseline = the oracle (a C restatement of Aer's QubitVector) timed on
           the host cores over a bounded sample of the same fused ops

``--impl reference`` times the reference's CPU algorithm (the oracle port;
the reference's own build does not exist on the GPU host) on the same
workload and metric.  The state (17 GB at complex128) exceeds L2 (129 MB),
so no L2 flush is needed between steps.
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

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            q = "clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
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

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=5)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 2 + i and "Active" in s[2 + i]
                          and not s[2 + i].startswith("Not")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_baseline(P, fused_ops, n_small, precision, budget_s=12.0):
    """Oracle (C restatement of Aer's QubitVector, OpenMP) on a bounded sample:
    the fused ops applied to a 2^n_small state on all host cores."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads, 14)
    o = O.OracleQV(n_small)
    # map the ops onto n_small qubits (qubit q -> q mod n_small, keeping them distinct)
    t0 = time.perf_counter()
    done = 0
    amp_bytes = 16 if precision == "double" else 8
    for q, m in fused_ops:
        qq = [x % n_small for x in q]
        if len(set(qq)) != len(qq):
            continue
        o.apply_matrix(qq, m)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    gbs = done * 2 * (1 << n_small) * amp_bytes / dt / 1e9
    return {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"{done} fused ops of the workload on a {n_small}-qubit complex128 state "
                      f"({(1 << n_small) * 16 / 1e9:.2f} GB), {dt:.1f} s, OpenMP {threads} threads"}


def run_reference_arm(args):
    """--impl reference: the reference's CPU algorithm (oracle port) on the
    same workload, all host threads, bounded per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    P = entry.load_package()
    from oracle import oracle as O

    O.build()
    qc = qv_circuit(P, args.qubits, args.layers, args.seed)
    segs, _, _, meta = P.AerSimulator(precision=args.precision).compile(qc)
    nc = segs[0][1]
    fused = [(q, nc.op_matrix(i)) for i, (_, _, q) in enumerate(nc.ops())]
    n_small = min(args.qubits, 26)
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(P, fused[:4], n_small, args.precision, budget_s=2.0)
    for _ in range(args.steps):
        vals.append(cpu_baseline(P, fused, n_small, args.precision, budget_s=10.0))
    v = float(np.median([x["value"] for x in vals]))
    base = vals[-1]
    line = {"metric": "fused-gate GB/s", "value": v, "unit": "GB/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "dtype": "c128" if args.precision == "double" else "c64", "data": "synthetic",
            "config": {"workload": f"QV {args.qubits}q x {args.layers} layers, Aer fusion max 5", "qubits": args.qubits},
            "cpu_baseline": {**base, "value": v}, "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0,
                                                         "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="double", choices=["double", "single"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--layers", type=int, default=30)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)

    import torch  # device sync / events and torch.distributed for N > 1

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    P = entry.load_package()
    P.build()
    L = P.lib()
    qc = qv_circuit(P, args.qubits, args.layers, args.seed)
    sim = P.AerSimulator(precision=args.precision)
    segs, _, _, meta = sim.compile(qc)
    nc = segs[0][1]
    ops = nc.ops()
    amp_bytes = 16 if args.precision == "double" else 8
    pass_bytes = 2 * (1 << args.qubits) * amp_bytes
    st = P.QubitVector(args.qubits, args.precision)
    stream_ptr = C.c_void_p()
    # time on the engine's own stream: events recorded around gbqv_execute
    torch.cuda.init()

    def step():
        A_check(L.gbqv_execute(st.handle, nc.handle), st)

    def A_check(rc, s):
        if rc != 0:
            raise RuntimeError(L.gbqv_last_error(s.handle).decode())

    st.initialize()
    for _ in range(args.warmup):
        step()
    st.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler()
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    st.synchronize()
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    t_step = dt / args.steps
    if world > 1:
        tt = torch.tensor([t_step], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_step = float(tt.item())
    value = len(ops) * pass_bytes / t_step / 1e9 * world

    # e2e through the public API: upload |psi0> from pinned host memory, run
    # the fused circuit, read back the 8-qubit marginal
    psi0 = np.zeros(1 << args.qubits, dtype=np.complex128) if args.qubits <= 30 else None
    e2e = None
    if psi0 is not None:
        psi0[0] = 1.0
        t1 = time.perf_counter()
        for _ in range(max(1, args.steps)):
            st.initialize_from_vector(psi0)
            step()
            st.probabilities(list(range(8)))
        st.synchronize()
        te = (time.perf_counter() - t1) / max(1, args.steps)
        e2e = {"value": round(len(ops) * pass_bytes / te / 1e9, 3), "unit": "GB/s",
               "h2d_bytes_per_step": int(psi0.nbytes), "d2h_bytes_per_step": 8 * 256}
    peak, peak_kind = hbm_peak()
    # dominant kernel: the fused-gate pass; per-launch bytes = one read+write of the state
    ms_per_launch = t_step * 1e3 / len(ops)
    achieved = pass_bytes / (ms_per_launch / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": None, "peak_kind": peak_kind}
    base = None
    if rank == 0 and not args.no_cpu_baseline:
        fused = [(q, nc.op_matrix(i)) for i, (_, _, q) in enumerate(ops)]
        base = cpu_baseline(P, fused, min(args.qubits, 26), args.precision)
    if rank == 0:
        line = {"metric": "fused-gate GB/s", "value": round(value, 3), "unit": "GB/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "c128" if args.precision == "double" else "c64", "data": "synthetic",
                "config": {"workload": f"QV {args.qubits}q x {args.layers} layers (450 Haar SU(4)), Aer fusion max 5",
                           "qubits": args.qubits, "layers": args.layers, "fused_ops": len(ops),
                           "l2": "state larger than L2, no flush"},
                "gpu_launches": None, "roofline": roof, "cpu_baseline": base, "e2e": e2e, "clocks": clk}
        print(json.dumps(line))
    st.close()


if __name__ == "__main__":
    main()

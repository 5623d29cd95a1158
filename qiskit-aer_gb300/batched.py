"""Batches of independent circuit instances of uneven size in one persistent
launch (gbqv_batch_* in include/gbqv.h): per instance the final-state shots,
<H> and the adjoint gradient.  ``config5_instances`` builds the seeded
workload of hardware-efficient ansatz instances (RY / RZ on every qubit plus
a linear CX ladder per layer) with random Pauli Hamiltonians."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as A

RX, RY, RZ, CX, CZ, H = range(6)


class Batch:
    def __init__(self, precision: str = "double"):
        self._L = A.lib()
        h = C.c_void_p()
        A.check(self._L.gbqv_batch_create(A.C128 if precision == "double" else A.C64, C.byref(h)))
        self._h = h
        self.instances = []

    def close(self):
        if getattr(self, "_h", None):
            self._L.gbqv_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, num_qubits, gates, params, terms, coeffs, shots, seed) -> int:
        """gates: [(kind, q0, q1, param_index or -1)], terms: [(qubits, label)]."""
        kinds = (C.c_int * max(1, len(gates)))(*[g[0] for g in gates])
        qs = np.ascontiguousarray(np.array([[g[1], g[2]] for g in gates], dtype=np.uint64).reshape(-1))
        pi = (C.c_int * max(1, len(gates)))(*[g[3] for g in gates])
        pa = np.ascontiguousarray(np.asarray(params, dtype=np.float64))
        tq, offs, labels = [], [0], []
        for q, lab in terms:
            tq.extend(int(x) for x in q)
            offs.append(len(tq))
            labels.append(lab.encode())
        tqa = np.ascontiguousarray(np.asarray(tq, dtype=np.uint64))
        oa = (C.c_int * len(offs))(*offs)
        la = (C.c_char_p * len(labels))(*labels)
        ca = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64))
        idx = C.c_int()
        A.check(self._L.gbqv_batch_add(self._h, int(num_qubits), len(gates), kinds, qs.ctypes.data_as(A.u64p), pi,
                                       pa.ctypes.data_as(A.dp), pa.size, len(terms), tqa.ctypes.data_as(A.u64p), oa,
                                       la, ca.ctypes.data_as(A.dp), int(shots), int(seed), C.byref(idx)))
        self.instances.append((num_qubits, len(params), int(shots)))
        return idx.value

    def set_teams(self, max_team_instances: int = 64, min_cost_fraction: float = 0.5) -> None:
        """Two CTAs for each of the costliest instances (gbqv_batch_set_teams);
        call before the first run."""
        A.check(self._L.gbqv_batch_set_teams(self._h, int(max_team_instances), float(min_cost_fraction)))

    def set_fp64(self, on: bool = True) -> None:
        """Complex128 arithmetic on the FP64 pipe instead of float pairs
        (gbqv_batch_set_fp64); call before the first run."""
        A.check(self._L.gbqv_batch_set_fp64(self._h, int(bool(on))))

    def run(self, want_grad: bool = True) -> float:
        ms = C.c_double()
        A.check(self._L.gbqv_batch_run(self._h, int(want_grad), C.byref(ms)))
        return ms.value

    def result(self, i: int):
        n, npar, shots = self.instances[i]
        e, lat = C.c_double(), C.c_double()
        g = np.zeros(npar, dtype=np.float64)
        s = np.zeros(shots, dtype=np.uint64)
        A.check(self._L.gbqv_batch_result(self._h, i, C.byref(e), g.ctypes.data_as(A.dp), npar,
                                          s.ctypes.data_as(A.u64p), shots, C.byref(lat)))
        return e.value, g, s, lat.value


def hea_gates(num_qubits: int, layers: int):
    """(kind, q0, q1, param) list of the hardware-efficient ansatz and its parameter count."""
    gates, p = [], 0
    for _ in range(layers):
        for q in range(num_qubits):
            gates.append((RY, q, q, p))
            p += 1
        for q in range(num_qubits):
            gates.append((RZ, q, q, p))
            p += 1
        for q in range(num_qubits - 1):
            gates.append((CX, q, q + 1, -1))
    return gates, p


def config5_instances(count: int, seed: int, qmin=12, qmax=22, dmin=4, dmax=16, tmin=20, tmax=60, shots=4096):
    """Seeded instances: n ~ U{qmin..qmax}, depth ~ U{dmin..dmax}, own theta,
    a tmin..tmax-term Pauli Hamiltonian of weight 1-4, `shots` shots."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(qmin, qmax + 1))
        depth = int(rng.integers(dmin, dmax + 1))
        gates, npar = hea_gates(n, depth)
        theta = rng.uniform(-np.pi, np.pi, npar)
        nt = int(rng.integers(tmin, tmax + 1))
        terms = []
        for _ in range(nt):
            w = int(rng.integers(1, min(4, n) + 1))
            q = sorted(int(x) for x in rng.choice(n, w, replace=False))
            terms.append((q, "".join(rng.choice(list("XYZ"), w))))
        coeffs = rng.normal(size=nt)
        out.append(dict(n=n, depth=depth, gates=gates, theta=theta, terms=terms, coeffs=coeffs, shots=shots,
                        seed=seed * 100003 + i))
    return out


def shard(instances, rank: int, world: int):
    """Indices of the instances rank `rank` of `world` runs: greedy balance of
    the per-instance cost (depth x 2^n), no data exchange between ranks."""
    cost = [inst["depth"] * (1 << inst["n"]) for inst in instances]
    load = [0] * world
    owner = [0] * len(instances)
    for i in sorted(range(len(instances)), key=lambda j: -cost[j]):
        r = min(range(world), key=lambda k: load[k])
        owner[i] = r
        load[r] += cost[i]
    return [i for i in range(len(instances)) if owner[i] == rank]


def run_sharded(instances, runner, group=None):
    """Run this rank's share with runner(list of instances) -> list of energies
    and all-gather the energies in instance order (torch.distributed; one
    gather of the results, nothing during the run)."""
    import torch
    import torch.distributed as dist

    rank, world = (dist.get_rank(group), dist.get_world_size(group)) if dist.is_initialized() else (0, 1)
    mine = shard(instances, rank, world)
    vals = runner([instances[i] for i in mine])
    out = torch.full((len(instances),), float("nan"), dtype=torch.float64)
    for i, v in zip(mine, vals):
        out[i] = v
    if world > 1:
        parts = [torch.empty_like(out) for _ in range(world)]
        dist.all_gather(parts, out, group=group)
        for p in parts:
            mask = ~torch.isnan(p)
            out[mask] = p[mask]
    return out.numpy()

"""Benchmark: atoms/s of energy + forces on one GB300.

Workload (the batched configuration the metric is quoted on): 4096 cubic
Li/Si/O cells with log-uniform atom counts in [16, 512] (~597k atoms),
Chebyshev descriptor radial order 10 (Rc 6.0) / angular order 4 (Rc 4.0),
species-weighted (32 features), one 32-32-32-1 tanh network per species,
random weights; synthetic data generated from a fixed seed.

A step is one full energy-and-force pass over the whole batch: neighbour
search, descriptors, networks, energies, adjoint forces.  The batched
mixed-precision path is timed (the headline) next to the plain FP64 path on
the same batch; the mixed-precision error against FP64 is reported.

Timing: W untimed warm-up steps, then K steps each bracketed by CUDA events
on the launching stream, with an L2 flush (a 512 MB write) between steps
outside the events; barrier + synchronize around the timed region; max over
ranks.  `e2e` repeats the measurement through the C-ABI host-buffer entry
point (aenet_gpu_batch_energy_forces) from pinned host memory, copies
included.  `cpu_baseline` times the FP64 oracle (a restatement of the
reference's predict.x loop, its linked-cell search included) on a bounded
sample on all host cores.

--impl reference times that CPU implementation instead (rank 0 only).
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "atoms/s E+F on 1 GB300: batched mixed-prec vs plain FP64 at ≤1 meV/atom"
WORKLOAD = ("lisio_batch_4096: 4096 cubic Li/Si/O cells, 16-512 atoms (log-uniform), "
            "0.08 atoms/A^3, Chebyshev r10/6.0 a4/4.0 (32 features), 32-32-32-1 x3, E+F")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nstruc", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--lanes-per-atom", type=int, default=0,
                    help="fix the descriptor kernels' lanes per atom (implies --no-tune)")
    ap.add_argument("--cell-div", type=int, default=0,
                    help="fix the neighbour grid's cells per cut-off (implies --no-tune)")
    ap.add_argument("--neighbour-kernel", default="", choices=["", "cell", "atom", "stream", "half", "struct", "struct_half"],
                    help="fix the neighbour-search kernel (implies --no-tune)")
    ap.add_argument("--z-refine", type=int, default=0,
                    help="search cells this many times narrower along the third axis")
    ap.add_argument("--angular-terms", default="moments", choices=["moments", "pairs"],
                    help="mixed-path angular Chebyshev terms (moment form or pair sums)")
    ap.add_argument("--no-md", action="store_true", help="skip the 1M-atom MD leg")
    ap.add_argument("--md-steps", type=int, default=100)
    ap.add_argument("--no-train", action="store_true", help="skip the training-step leg")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the single-structure configurations (256, 4000, 9000, 1M atoms)")
    ap.add_argument("--cache", default=os.path.join(tempfile.gettempdir(), "aenet_gb300_bench"))
    return ap.parse_args()


# ----------------------------------------------------------------- workload
def load_workload(args, rank):
    """The seeded batch; cached (structures and network weights) on disk
    because the random placement takes a few seconds."""
    from aenet_gb300 import nnfile, workloads
    from aenet_gb300.replicas import replica_seed
    seed = replica_seed(args.seed, rank)
    os.makedirs(args.cache, exist_ok=True)
    f = os.path.join(args.cache, "lisio_%d_%d.npz" % (seed, args.nstruc))
    if os.path.exists(f):
        z = np.load(f)
        nat = z["natoms"]
        offs = np.concatenate([[0], np.cumsum(nat)])
        structs = [workloads.Structure(z["pos"][offs[k]:offs[k + 1]],
                                       z["typ"][offs[k]:offs[k + 1]], z["cells"][k])
                   for k in range(len(nat))]
        types = ["Li", "Si", "O"]
        arch = [32, 32, 32, 1]
        w = workloads.Workload("lisio_batch_4096", types,
                               workloads.cheb_setups(types, 10, 6.0, 4, 4.0), arch, structs, seed)
        w.networks = {t: nnfile.make_network(arch, z["W_" + t]) for t in types}
        return w
    w = workloads.lisio_batch_4096(seed=seed, nstruc=args.nstruc)
    nat, pos, typ, cells, _ = w.packed()
    tmp = f + ".tmp%d.npz" % os.getpid()
    np.savez(tmp, natoms=nat, pos=pos, typ=typ, cells=cells,
             **{"W_" + t: w.networks[t]["W"] for t in w.types})
    os.replace(tmp, f)
    return w


# ----------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 8]
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[4 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ----------------------------------------------------------------- helpers
def neighbour_stats(plan, a_rc, r_rc):
    import torch
    cap, cnt, jt, vec = plan.neighbors()
    d = vec[..., 3]
    valid = torch.arange(cap, device=d.device)[None, :] < cnt[:, None].long()
    nr = ((d <= r_rc) & (d > 1e-12) & valid).sum(1).double()
    na = ((d <= a_rc) & (d >= 1e-12) & valid).sum(1).double()
    P = na * (na - 1) / 2
    return {"n_r": nr.mean().item(), "n_a": na.mean().item(), "P": P.mean().item(),
            "n_all": cnt.double().mean().item(), "cap": cap, "n_max": int(cnt.max().item())}


def cheb_flops(nb, R, A, nsf, m, arch):
    """Per-atom flop counts of the reference's pair-form algorithm (radial
    terms per neighbour, angular terms per pair): the moment form does
    fewer, so FP32 rates computed from these are effective rates."""
    nr, na, P = nb["n_r"], nb["n_a"], nb["P"]
    fwd = nr * (16 + (5 + 2 * (m - 1)) * R) + 6 * na + P * (9 + (5 + 2 * (m - 1)) * A) + 2 * nsf
    adj = nr * (12 + (9 + 2 * (m - 1)) * R) + P * (77 + (8 + 2 * (m - 1)) * A)
    mlp_f = sum(2 * arch[l] * arch[l + 1] + arch[l + 1] for l in range(len(arch) - 1))
    mlp_b = sum(2 * arch[l] * arch[l + 1] + 2 * arch[l + 1] for l in range(len(arch) - 1))
    return {"descriptor": fwd, "adjoint": adj, "networks": mlp_f + mlp_b}


def oracle_descriptor_fn(oracle):
    def fn(workload, paths, ids):
        oracle.load(workload.types, paths)
        rows, spec = [], []
        ids = set(int(i) for i in ids)
        off = 0
        for s in workload.structures:
            local = [i - off for i in range(off, off + s.natoms) if i in ids]
            off += s.natoms
            if not local:
                continue
            _, centres, nb = oracle.neighbors(s.cell, s.positions, s.types, atoms=local)
            for q, a in enumerate(local):
                rows.append(oracle.descriptor(centres[a], int(s.types[a]), nb[q][0], nb[q][3],
                                              scaled=False))
                spec.append(int(s.types[a]))
        return np.array(rows), np.array(spec)
    return fn


def time_oracle(oracle, structures, threads):
    t0 = time.perf_counter()
    n = 0
    for s in structures:
        oracle.structure(s.cell, s.positions, s.types, nthreads=threads)
        n += s.natoms
    return n, time.perf_counter() - t0


def pick_sample(oracle, structures, threads, seconds):
    """Leading structures of the batch whose oracle time is about `seconds`."""
    probe = structures[:8]
    n, dt = time_oracle(oracle, probe, threads)
    per_atom = dt / max(n, 1)
    budget = seconds / max(per_atom, 1e-9)
    out, tot = [], 0
    for s in structures:
        if tot + s.natoms > budget and out:
            break
        out.append(s)
        tot += s.natoms
    return out


# ----------------------------------------------------------------- arms
def run_reference(args):
    """The reference's CPU algorithm (oracle port) on the host cores."""
    from oracle import Oracle
    from aenet_gb300 import workloads
    w = load_workload(args, 0)
    d = tempfile.mkdtemp(prefix="aenet_ref_")
    o = Oracle()
    paths = workloads.write_potentials(w, d, oracle_descriptor_fn(o), max_atoms_for_stats=4000)
    o.load(w.types, paths)
    o.set_candidates("cells")
    threads = os.cpu_count() or 1
    per_step = max(2.0, args.cpu_seconds * 4 / max(args.steps + args.warmup, 1))
    sample = pick_sample(o, w.structures, threads, per_step)
    for _ in range(args.warmup):
        time_oracle(o, sample, threads)
    times, atoms = [], 0
    for _ in range(args.steps):
        n, dt = time_oracle(o, sample, threads)
        times.append(dt)
        atoms = n
    ms = 1e3 * float(np.mean(times))
    value = atoms / (ms * 1e-3)
    desc = ("first %d of %d cells (%d atoms) per step, FP64 oracle port of predict.x "
            "(linked-cell search as written), %d OpenMP threads" % (len(sample), len(w.structures),
                                                                     atoms, threads))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "atoms/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "sample": desc, "precision": "fp64"},
            "cpu_baseline": {"value": value, "unit": "atoms/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": "atoms/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from aenet_gb300 import _lib, workloads
    from aenet_gb300.core import ANNPotentials, FP64, MIXED
    from aenet_gb300.plan import Plan

    w = load_workload(args, rank)
    d = tempfile.mkdtemp(prefix="aenet_bench_")
    paths = workloads.write_potentials(w, d, workloads.gpu_descriptor_fn)
    ann = ANNPotentials(paths)
    nat, pos, typ, cells, pbc = w.packed()
    N, S = int(nat.sum()), len(nat)
    dev = torch.device("cuda", local)
    p = torch.tensor(pos, device=dev)
    t = torch.tensor(typ, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    tuned = None
    from aenet_gb300 import core as _core
    _core.set_option("angular_terms", args.angular_terms)
    if args.lanes_per_atom or args.cell_div or args.neighbour_kernel or args.z_refine:
        args.no_tune = True
        if args.z_refine:
            _core.set_option("z_refine", args.z_refine)
        if args.lanes_per_atom:
            _core.set_option("lanes_per_atom", args.lanes_per_atom)
        if args.cell_div:
            _core.set_option("cell_div", args.cell_div)
        if args.neighbour_kernel:
            _core.set_option("neighbour_kernel", args.neighbour_kernel)
        tuned = {"lanes_per_atom": args.lanes_per_atom or None, "cell_div": args.cell_div or None,
                 "z_refine": args.z_refine or None,
                 "neighbour_kernel": args.neighbour_kernel or None, "fixed": True}
    if not args.no_tune:
        from aenet_gb300 import autotune
        tuned = autotune.tune(nat, cells, pbc, pos, typ, precision=MIXED, cache=None)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    def timed(plan, out, steps, graph):
        fn = (lambda: graph.replay()) if graph is not None else (lambda: plan.run(p, t, out=out))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        barrier()
        wall0 = time.perf_counter()
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            fn()
            ev[k][1].record(stream)
        barrier()
        wall = time.perf_counter() - wall0
        ms = [a.elapsed_time(b) for a, b in ev]
        return float(np.sum(ms)), wall

    def prepare(prec):
        plan = Plan(nat, cells, pbc, precision=prec, coords0=pos)
        out = plan.run(p, t)
        plan.check()
        for _ in range(args.warmup):
            plan.run(p, t, out=out)
        torch.cuda.synchronize()
        graph = None
        if not args.no_graph:
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                plan.run(p, t, out=out)
            for _ in range(max(1, args.warmup)):
                graph.replay()
            torch.cuda.synchronize()
        return plan, out, graph

    # ---- mixed precision (headline)
    plan32, out32, g32 = prepare(MIXED)
    sampler = ClockSampler(local)
    sampler.start()
    total_ms, wall = timed(plan32, out32, args.steps, g32)
    clocks = sampler.stop()
    plan32.check()
    from aenet_gb300.replicas import job_rate, max_over_ranks
    # every rank evaluates its own batch: total atoms over the slowest rank
    value = job_rate(N, total_ms * 1e-3 / args.steps, device=dev)
    total_ms = max_over_ranks(total_ms, device=dev)
    ms_step = total_ms / args.steps
    res32 = {k: v.clone() for k, v in out32.items()}

    # ---- stage profile and roofline of the dominant kernel
    stages = {}
    for _ in range(3):
        prof = plan32.profile(p, t)
        for k, v in prof.items():
            stages[k] = stages.get(k, 0.0) + v / 3
    sp = w.setups["Li"]
    r_rc, r_ord, a_rc, a_ord = sp["sfparam"][0]
    nb = neighbour_stats(plan32, a_rc, r_rc)
    R, A = int(r_ord) + 1, int(a_ord) + 1
    fl = cheb_flops(nb, R, A, sp["nsf"], 2, w.arch)
    peak = C.c_double(0.0)
    _lib.lib().aenet_gpu_measure_fp32_peak(C.byref(peak), C.c_void_p(stream.cuda_stream))
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
    # Per-kernel rooflines.  k_neighbors: HBM bound, the algorithmic bytes
    # B_nl = 3 w + 4 + 16 + 8 n per atom (FP64 positions read, type, cell
    # id / key / value, a neighbour index written and read back per pair),
    # over the search kernel's own CUDA-event time.  Descriptor and adjoint:
    # the FP32 pipe with the pair-form flop counts per atom (the moment form
    # does fewer flops, so these are effective rates).  Networks: tensor
    # pipe, reported as FP32-equivalent rates of the same flop counts.
    nsf = sp["nsf"]
    hbm = peaks.get("hbm_gbs")
    b_nl = 3 * 8 + 4 + 16 + 8 * nb["n_all"]
    traffic_per_atom = {}
    tf = os.path.join(ROOT, "profiles", "traffic_per_atom.txt")
    if os.path.exists(tf):
        traffic_per_atom = json.load(open(tf))
    limiters = {}
    lf = os.path.join(ROOT, "profiles", "limiters_lisio_batch_1024.txt")
    if os.path.exists(lf):
        limiters = json.load(open(lf))
    times = {"k_neighbors": stages["neighbour_search"], "k_cheb_forward": stages["descriptor"],
             "k_cheb_adjoint": stages["adjoint"], "k_mlp_tc": stages["networks"]}
    kernels_roof = {}
    for k, ms_k in times.items():
        if k == "k_neighbors":
            ach = b_nl * N / (ms_k * 1e-3) / 1e9
            r = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                 "frac": ach / hbm, "bytes_per_atom": b_nl,
                 "bytes_formula": "3*8 + 4 + 16 + 8*n_all per atom (n_all = %.2f)" % nb["n_all"]}
            alg = b_nl * N
        else:
            f = {"k_cheb_forward": fl["descriptor"], "k_cheb_adjoint": fl["adjoint"],
                 "k_mlp_tc": fl["networks"]}[k]
            ach = f * N / (ms_k * 1e-3) / 1e12
            r = {"bound": "fp32" if k != "k_mlp_tc" else "tensor", "achieved": ach,
                 "peak": peak.value, "unit": "TFLOP/s",
                 "frac": ach / peak.value if peak.value else None, "flops_per_atom": f,
                 "peak_source": "measured live: FP32 FMA throughput kernel on this GPU"}
            alg = None
        r["ms_per_launch"] = ms_k
        tpa = traffic_per_atom.get(k)
        r["traffic"] = None if tpa is None else tpa * N
        if tpa is not None and alg:
            r["traffic_over_algorithmic"] = tpa * N / alg
        if limiters.get(k):
            r["limiter"] = dict(limiters[k], source="profiles/ncu_full_lisio_batch_1024.md")
        kernels_roof[k] = r
    dom = max(times, key=lambda k: times[k])
    roof = dict(kernels_roof[dom], kernel=dom)
    roof["other_kernels"] = {k: {q: v for q, v in r.items() if q in ("bound", "achieved", "frac",
                                                                     "unit", "ms_per_launch")}
                             for k, r in kernels_roof.items() if k != dom}
    plan32.close()

    # ---- plain FP64 path on the same batch
    plan64, out64, g64 = prepare(FP64)
    ms64, _ = timed(plan64, out64, max(1, args.fp64_steps), g64)
    ms64 /= max(1, args.fp64_steps)
    value64 = job_rate(N, ms64 * 1e-3, device=dev)
    natoms_t = torch.tensor(nat, device=dev, dtype=torch.float64)
    dE = ((res32["E"] - out64["E"]).abs() / natoms_t)
    dF = res32["F"] - out64["F"]
    errors = {"energy_max_eV_per_atom": dE.max().item(),
              "energy_mean_eV_per_atom": dE.mean().item(),
              "force_rms_eV_per_A": dF.pow(2).mean().sqrt().item(),
              "force_max_eV_per_A": dF.abs().max().item(),
              "force_scale_rms_eV_per_A": out64["F"].pow(2).mean().sqrt().item()}
    plan64.close()

    # ---- e2e through the C-ABI with host buffers (pinned)
    e2e = None
    if not args.no_e2e:
        lib = _lib.lib()
        hp = torch.empty((N, 3), dtype=torch.float64, pin_memory=True)
        hp.copy_(torch.from_numpy(pos))
        ht = torch.empty(N, dtype=torch.int32, pin_memory=True)
        ht.copy_(torch.from_numpy(typ))
        hF = torch.empty((N, 3), dtype=torch.float64, pin_memory=True)
        hE = torch.empty(S, dtype=torch.float64, pin_memory=True)
        nat_c = np.ascontiguousarray(nat, dtype=np.int32)
        cells_c = np.ascontiguousarray(cells.reshape(S, 9))
        pbc_c = np.ascontiguousarray(pbc, dtype=np.int32)
        st = C.c_int(0)

        def call():
            lib.aenet_gpu_batch_energy_forces(
                S, nat_c.ctypes.data_as(C.c_void_p), C.c_void_p(hp.data_ptr()),
                C.c_void_p(ht.data_ptr()), cells_c.ctypes.data_as(C.c_void_p),
                pbc_c.ctypes.data_as(C.c_void_p), MIXED, C.c_void_p(hE.data_ptr()),
                C.c_void_p(hF.data_ptr()), None, C.byref(st))
            if st.value:
                raise RuntimeError("aenet_gpu_batch_energy_forces status %d" % st.value)

        for _ in range(max(1, args.warmup)):
            call()
        calls = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            call()
            calls.append(time.perf_counter() - t0)
        e2e_s = float(np.mean(calls))
        e2e_rate = job_rate(N, e2e_s, device=dev)
        tt = torch.tensor([max_over_ranks(e2e_s, device=dev)], dtype=torch.float64)
        e2e = {"value": e2e_rate, "unit": "atoms/s",
               "h2d_bytes_per_step": N * 24 + N * 4, "d2h_bytes_per_step": S * 8 + N * 24,
               "ms_per_step": 1e3 * tt.item(), "api": "aenet_gpu_batch_energy_forces"}
        # same kernels, neighbour order within a cell may differ: FP32 noise
        dev_e = np.abs(hE.numpy() - res32["E"].cpu().numpy()) / nat
        assert dev_e.max() < 1e-5, dev_e.max()
        # cold calls: every call brings a batch layout the previous call did
        # not have (the structures alternately in their order and reversed),
        # so the cached plans are rebuilt and their graphs captured anew
        offs = np.concatenate([[0], np.cumsum(nat)])
        rev = np.arange(S)[::-1]
        layouts = []
        for order in (np.arange(S), rev):
            idx = np.concatenate([np.arange(offs[k], offs[k + 1]) for k in order])
            hp_o = torch.empty((N, 3), dtype=torch.float64, pin_memory=True)
            hp_o.copy_(torch.from_numpy(np.ascontiguousarray(pos[idx])))
            ht_o = torch.empty(N, dtype=torch.int32, pin_memory=True)
            ht_o.copy_(torch.from_numpy(np.ascontiguousarray(typ[idx])))
            layouts.append((np.ascontiguousarray(nat[order], dtype=np.int32), hp_o, ht_o,
                            np.ascontiguousarray(cells[order].reshape(S, 9)),
                            np.ascontiguousarray(pbc[order], dtype=np.int32)))

        def call_layout(L):
            n_o, hp_o, ht_o, c_o, p_o = L
            lib.aenet_gpu_batch_energy_forces(
                S, n_o.ctypes.data_as(C.c_void_p), C.c_void_p(hp_o.data_ptr()),
                C.c_void_p(ht_o.data_ptr()), c_o.ctypes.data_as(C.c_void_p),
                p_o.ctypes.data_as(C.c_void_p), MIXED, C.c_void_p(hE.data_ptr()),
                C.c_void_p(hF.data_ptr()), None, C.byref(st))
            if st.value:
                raise RuntimeError("aenet_gpu_batch_energy_forces status %d" % st.value)

        cold = []
        ncold = max(3, args.steps // 4)
        for k in range(ncold + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            call_layout(layouts[(k + 1) % 2])
            if k:   # the first alternation only leaves the warm layout
                cold.append(time.perf_counter() - t0)
        cold_s = float(np.mean(cold))
        e2e["cold"] = {"value": job_rate(N, cold_s, device=dev), "unit": "atoms/s",
                       "ms_per_step": 1e3 * cold_s, "calls": len(cold),
                       "note": "each call a new batch layout (structure order alternated): "
                               "plans and graphs rebuilt inside the timed call"}

    # ---- CPU baseline (rank 0): the oracle port on a bounded sample
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import Oracle
        o = Oracle()
        o.load(w.types, paths)
        o.set_candidates("cells")
        threads = os.cpu_count() or 1
        sample = pick_sample(o, w.structures, threads, args.cpu_seconds)
        n, dt = time_oracle(o, sample, threads)
        s1 = pick_sample(o, w.structures, 1, args.cpu_seconds / 5)
        n1, dt1 = time_oracle(o, s1, 1)
        cpu = {"value": n / dt, "unit": "atoms/s", "cores": threads, "kind": "port",
               "sample": "first %d of %d cells (%d atoms), FP64 oracle port of predict.x "
                         "(linked-cell search as written), %d OpenMP threads, %.1f s"
                         % (len(sample), S, n, threads, dt),
               "one_thread": {"value": n1 / dt1, "sample_atoms": n1, "seconds": dt1}}
        o.close()

    # ---- training step on the same batch: loss E + F and its weight gradient
    # against targets of an FP64 teacher potential of the same shape (random
    # networks from seed 104, the batch's descriptor normalisation)
    train = None
    if not args.no_train:
        from aenet_gb300 import nnfile
        from aenet_gb300.plan import LOSS_ENERGY_FORCES
        stats = {}
        for tname in w.types:
            _, stp_t, _, _ = nnfile.read_nn(paths[tname])
            stats[tname] = (stp_t["sfval_min"], stp_t["sfval_max"], stp_t["sfval_avg"],
                            stp_t["sfval_cov"])
        teacher_nets = workloads.glorot_networks(np.random.default_rng(104), w.types, w.arch)
        tpaths = workloads.write_potentials(w, tempfile.mkdtemp(prefix="aenet_teacher_"),
                                            stats=stats, networks=teacher_nets)
        ann.release()
        tann = ANNPotentials(tpaths)
        plan_e = Plan(nat, cells, pbc, precision=FP64, coords0=pos)
        tout = plan_e.run(p, t)
        plan_e.check()
        E_t, F_t = tout["E"].clone(), tout["F"].clone()
        plan_e.close()
        tann.release()
        ann = ANNPotentials(paths)
        plan_t = Plan(nat, cells, pbc, precision=MIXED, coords0=pos)
        gbuf = torch.empty(ann.nweights(), dtype=torch.float64, device=dev)
        lbuf = torch.empty(1, dtype=torch.float64, device=dev)

        def tstep():
            plan_t.loss_gradient(p, t, E_t, F_t, mode=LOSS_ENERGY_FORCES, w_E=1.0, w_F=0.1,
                                 grad=gbuf, loss=lbuf)

        for _ in range(max(1, args.warmup)):
            tstep()
        plan_t.check()
        tgraph = None
        if not args.no_graph:
            tgraph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(tgraph):
                tstep()
            tgraph.replay()
            torch.cuda.synchronize()
        tms = []
        for _ in range(max(3, args.steps // 4)):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            if tgraph is not None:
                tgraph.replay()
            else:
                tstep()
            b.record(stream)
            b.synchronize()
            tms.append(a.elapsed_time(b))
        plan_t.check()
        tm = float(np.mean(tms))
        train = {"workload": "same batch: loss w_E sum (E-E_t)^2/N^2 + w_F sum |F-F_t|^2, "
                             "w_E 1, w_F 0.1, targets from an FP64 teacher potential of the same "
                             "shape (seed 104), gradient with respect to all %d weights"
                             % ann.nweights(),
                 "atoms_per_s": N / (tm * 1e-3), "ms_per_step": tm, "precision": "mixed",
                 "cuda_graph": tgraph is not None, "loss": float(lbuf.item())}
        del tgraph
        plan_t.close()

    ann.release()
    configs = None
    if rank == 0 and not args.no_configs:
        configs = run_configs(args, local, flush, peak.value)
    md = None
    if rank == 0 and not args.no_md:
        md = run_md(args, local)

    # the neighbour search: one kernel per structure block, which checks
    # the type ids and builds its own cell lists, when the plan takes the
    # per-structure search (at least twice as many structures as SMs);
    # otherwise the type check, binning, three scan kernels, scatter and the
    # search.  Then descriptor, 3 species-partition kernels, tensor-core
    # networks, the energy reduction (one kernel when every structure fits
    # one 2,048-atom chunk, else two), adjoint, force output.
    nb_kernel = (tuned or {}).get("neighbour_kernel") or args.neighbour_kernel or "atom"
    per_struct = nb_kernel in ("struct", "struct_half") and \
        len(nat) >= 2 * torch.cuda.get_device_properties(local).multi_processor_count
    energy_kernels = 1 if int(np.max(nat)) <= 2048 and int(np.min(nat)) >= 1 else 2
    launches_per_step = (1 if per_struct else 7) + 1 + 3 + 1 + energy_kernels + 1 + 1
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "atoms/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic (seeded structures, random-weight networks)",
                "config": {"workload": WORKLOAD, "nstruc": S, "natoms": N,
                           "precision": "mixed: fp32 descriptors/networks/forces, fp64 "
                                        "normalisation shift and per-structure energy sums",
                           "l2": "512 MB write between timed steps (outside the events); "
                                 "per-step working set > 1 GB",
                           "parallelism": "replicas" if world > 1 else "single GPU",
                           "cuda_graph": not args.no_graph,
                           "angular_terms": args.angular_terms,
                           "launch_shape": {k: v for k, v in (tuned or {}).items()
                                            if k != "all"}},
                "configs": configs, "md": md, "train_step": train,
                "neighbours": nb, "stages_ms": stages, "roofline": roof, "cpu_baseline": cpu,
                "e2e": e2e, "gpu_launches": launches_per_step * args.steps, "clocks": clocks,
                "wall_s_timed_region": wall,
                # the metric's own comparison last, so that it ends the line
                "fp64": {"value": value64, "unit": "atoms/s", "ms_per_step": ms64},
                "errors_vs_fp64": errors, "mixed_over_fp64": value / value64}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def behler_counts(plan, rc):
    """n (neighbours within rc) and P3 (pairs j < k of them with r_jk < rc
    too) per atom, averaged, from the plan's neighbour table."""
    import torch
    cap, cnt, jt, vec = plan.neighbors()
    n_tot, p3_tot = 0.0, 0.0
    for a0 in range(0, plan.natoms, 1024):
        v = vec[a0:a0 + 1024].double()
        c = cnt[a0:a0 + 1024].long()
        ok = (torch.arange(cap, device=v.device)[None, :] < c[:, None]) & (v[..., 3] < rc) \
            & (v[..., 3] > 1e-8)
        n_tot += ok.sum().item()
        R = v[..., :3]
        d = torch.cdist(R, R)
        m = ok[:, :, None] & ok[:, None, :] & (d < rc)
        p3_tot += (torch.triu(m, diagonal=1)).sum().item()
    return n_tot / plan.natoms, p3_tot / plan.natoms


def behler_flops(n, P3, g2, g4, nsf):
    """Canonical flops per atom of the G2/G4 forward and adjoint."""
    fwd = n * (14 + 10 * g2) + P3 * (30 + 16 * g4) + 2 * nsf
    adj = n * (9 + 8 * g2) + P3 * (40 + 40 * g4)
    return fwd, adj


def time_cpu(o, s, threads, seconds):
    """atoms/s of the oracle's predict.x loop on `threads` host threads over
    the first atoms of structure s (sized to about `seconds`)."""
    probe = min(s.natoms, 16 * threads)
    t0 = time.perf_counter()
    o.structure(s.cell, s.positions, s.types, nthreads=threads, atom_limit=probe)
    dt = time.perf_counter() - t0
    k = int(min(s.natoms, max(probe, probe * seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    o.structure(s.cell, s.positions, s.types, nthreads=threads, atom_limit=k)
    dt = time.perf_counter() - t0
    return k / dt, k


def per_atom_leg(w, paths, s):
    """The predict.x calling pattern through the libaenet C-ABI: one
    aenet_atomic_energy_and_forces call per atom with its neighbour list
    (lcl_nbdist_cart order), host arrays in and out, against the same calls
    of the oracle port on one host thread."""
    from aenet_gb300 import _lib
    from oracle import Oracle
    lib = _lib.lib()
    o = Oracle()
    o.load(w.types, paths)
    _, centres, nb = o.neighbors(s.cell, s.positions, s.types)
    n = s.natoms
    rows = []
    for i in range(n):
        nbcoo, _, nbl, nbt = nb[i]
        rows.append((np.ascontiguousarray(centres[i]), int(s.types[i]), i + 1, len(nbl),
                     np.ascontiguousarray(nbcoo), np.ascontiguousarray(nbt, dtype=np.int32),
                     np.ascontiguousarray(nbl, dtype=np.int32)))
    F = np.zeros((n, 3))
    E = C.c_double()
    st = C.c_int()

    def gpu_pass_rows():
        F[:] = 0.0
        etot = 0.0
        for ci, ti, ii, m, co, ty, ix in rows:
            lib.aenet_atomic_energy_and_forces(
                ci.ctypes.data_as(C.c_void_p), ti, ii, m, co.ctypes.data_as(C.c_void_p),
                ty.ctypes.data_as(C.c_void_p), ix.ctypes.data_as(C.c_void_p), n, C.byref(E),
                F.ctypes.data_as(C.c_void_p), C.byref(st))
            if st.value:
                raise RuntimeError("aenet_atomic_energy_and_forces status %d" % st.value)
            etot += E.value
        return etot

    gpu_pass_rows()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        e_gpu = gpu_pass_rows()
    dt_gpu = (time.perf_counter() - t0) / reps
    Fo = np.zeros((n, 3))
    t0 = time.perf_counter()
    e_cpu = 0.0
    for ci, ti, ii, m, co, ty, ix in rows:
        e_cpu += o.atomic_energy_and_forces(ci, ti, ii, co, ty, ix, Fo)
    dt_cpu = time.perf_counter() - t0
    o.close()
    return {"api": "aenet_atomic_energy_and_forces (one call per atom, host arrays)",
            "us_per_call": 1e6 * dt_gpu / n, "atoms_per_s": n / dt_gpu,
            "cpu_1_thread_us_per_call": 1e6 * dt_cpu / n, "cpu_1_thread_atoms_per_s": n / dt_cpu,
            "speedup_vs_cpu_1_thread": dt_cpu / dt_gpu,
            "energy_diff_eV": abs(e_gpu - e_cpu), "force_max_diff_eV_per_A": float(np.abs(F - Fo).max())}


def run_configs(args, local, flush, fp32_peak):
    """Energy and forces of the single-structure configurations, FP64 and
    mixed, device-timed (CUDA graph replays, L2 flushed between steps), the
    mixed path's error against FP64, and the oracle port of the reference's
    predict.x loop on 1 host thread and on all of them."""
    import torch
    from aenet_gb300 import workloads
    from aenet_gb300.core import ANNPotentials, FP64, MIXED
    from aenet_gb300.plan import Plan
    from oracle import Oracle
    stream = torch.cuda.current_stream()
    dev = torch.device("cuda", local)
    threads = os.cpu_count() or 1
    out = {}
    for name in ("cu_fcc_256", "aucu_fcc_4000", "tio2_rutile_9000", "cuau_fcc_1m"):
        w = workloads.WORKLOADS[name]()
        s = w.structures[0]
        d = tempfile.mkdtemp(prefix="aenet_cfg_")
        paths = workloads.write_potentials(w, d, workloads.gpu_descriptor_fn,
                                           max_atoms_for_stats=4000)
        ann = ANNPotentials(paths)
        behler = name.startswith("tio2")
        row = {"atoms": s.natoms}
        try:
            p = torch.tensor(s.positions, device=dev)
            t = torch.tensor(s.types, device=dev)
            res = {}
            for prec, key in ((FP64, "fp64"), (MIXED, "mixed")):
                plan = Plan([s.natoms], s.cell[None], [1], precision=prec, coords0=s.positions)
                o = plan.run(p, t, virial=behler)
                plan.check()
                graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(graph):
                    plan.run(p, t, virial=behler, out=o)
                for _ in range(3):
                    graph.replay()
                reps = 5 if s.natoms > 100000 or (behler and prec == FP64) else 20
                ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                      for _ in range(reps)]
                torch.cuda.synchronize()
                for k in range(reps):
                    flush.zero_()
                    ev[k][0].record(stream)
                    graph.replay()
                    ev[k][1].record(stream)
                torch.cuda.synchronize()
                ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
                plan.check()
                res[key] = {k2: v.clone() for k2, v in o.items()}
                row[key] = {"atoms_per_s": s.natoms / (ms * 1e-3), "ms": ms}
                if behler:
                    st = {}
                    for _ in range(3):
                        for k2, v in plan.profile(p, t).items():
                            st[k2] = st.get(k2, 0.0) + v / 3
                    row[key]["stages_ms"] = {k2: round(v, 4) for k2, v in st.items()}
                    if prec == FP64:
                        n_b, p3 = behler_counts(plan, 6.5)
                        nsf = w.setups[w.types[0]]["nsf"]
                        fwd, adj = behler_flops(n_b, p3, 8, 16, nsf)
                        row["behler"] = {"n": n_b, "P3": p3, "flops_fwd_per_atom": fwd,
                                         "flops_adj_per_atom": adj}
                del graph
                plan.close()
            if name == "cu_fcc_256":
                row["per_atom_api"] = per_atom_leg(w, paths, s)
            dE = abs(res["mixed"]["E"] - res["fp64"]["E"]).item() / s.natoms
            dF = res["mixed"]["F"] - res["fp64"]["F"]
            row["mixed_over_fp64"] = row["mixed"]["atoms_per_s"] / row["fp64"]["atoms_per_s"]
            row["errors_vs_fp64"] = {"energy_eV_per_atom": dE,
                                     "force_rms_eV_per_A": dF.pow(2).mean().sqrt().item(),
                                     "force_max_eV_per_A": dF.abs().max().item()}
            if behler:
                b = row["behler"]
                for key in ("fp64", "mixed"):
                    stg = row[key]["stages_ms"]
                    b[key + "_tflops_fwd"] = b["flops_fwd_per_atom"] * s.natoms / (
                        stg["descriptor"] * 1e-3) / 1e12
                    b[key + "_tflops_adj"] = b["flops_adj_per_atom"] * s.natoms / (
                        stg["adjoint"] * 1e-3) / 1e12
                if fp32_peak:
                    b["fp32_peak_tflops"] = fp32_peak
                    b["mixed_frac_fwd"] = b["mixed_tflops_fwd"] / fp32_peak
                    b["mixed_frac_adj"] = b["mixed_tflops_adj"] / fp32_peak
        finally:
            ann.release()
        if not args.no_cpu:
            o = Oracle()
            o.load(w.types, paths)
            o.set_candidates("cells")
            r1, k1 = time_cpu(o, s, 1, args.cpu_seconds / 8)
            ra, ka = time_cpu(o, s, threads, args.cpu_seconds / 8)
            o.close()
            row["cpu"] = {"1_thread": r1, "all_threads": ra, "threads": threads,
                          "sample_atoms": [k1, ka],
                          "kind": "port (FP64 oracle, predict.x loop, linked-cell search)"}
            row["mixed_over_cpu_all"] = row["mixed"]["atoms_per_s"] / ra
        out[name] = row
    return out


def run_md(args, local):
    """1,048,576-atom Cu/Au FCC (25% Au), 100 velocity-Verlet steps of 2 fs
    from Maxwell-Boltzmann velocities at 600 K, Verlet skin 0.3 A, mixed
    precision, with the FP64 energy of the same positions every 10 steps."""
    import torch
    from aenet_gb300 import workloads
    from aenet_gb300.core import ANNPotentials, MIXED
    from aenet_gb300.md import MolecularDynamics
    w = workloads.cuau_fcc_1m()
    d = tempfile.mkdtemp(prefix="aenet_md_")
    paths = workloads.write_potentials(w, d, workloads.gpu_descriptor_fn)
    ann = ANNPotentials(paths)
    s = w.structures[0]
    try:
        tuned = None
        if not args.no_tune:
            from aenet_gb300 import autotune
            tuned = autotune.tune(np.array([s.natoms]), s.cell[None], np.array([1]), s.positions,
                                  s.types, precision=MIXED, cache=None)
        md = MolecularDynamics(ann, s.positions, s.types, s.cell, velocities=w.velocities,
                               dt=2.0, skin=0.3, precision=MIXED)
        e0 = md.E_pot + md.E_kin
        md.run(2)    # warm-up (lazy allocations, first refresh)
        steps0, builds0 = md.counters()
        block = 10
        run_s, monitor, drift = 0.0, [], []
        for _ in range(max(1, args.md_steps // block)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ep, ek = md.run(block)
            run_s += time.perf_counter() - t0
            monitor.append(abs(md.energy_fp64() - ep) / s.natoms)
            drift.append(abs(ep + ek - e0) / s.natoms)
        steps, builds = md.counters()
        nsteps = steps - steps0
        bm, bn, rm, rn = md.phase_times()
        _, _, Fmd = md.state()
        force_rms = float(np.sqrt(np.mean(Fmd ** 2)))
        out = {"workload": "cuau_fcc_1m: 64^3 conventional FCC cells, a = 3.70 A, 25% Au, "
                           "sigma 0.1 A, Chebyshev r16/6.0 a8/4.0 (52 features), 52-20-20-1 x2",
               "atoms": s.natoms, "steps": int(nsteps), "dt_fs": 2.0, "skin_A": 0.3,
               "precision": "mixed forces, fp64 integration",
               "atom_steps_per_s": s.natoms * nsteps / run_s, "ms_per_step": 1e3 * run_s / nsteps,
               "neighbour_builds": int(builds - builds0),
               "force_part_ms_per_step": {
                   "with_table_build": bm / bn if bn else None, "build_steps": int(bn),
                   "with_refresh": rm / rn if rn else None, "refresh_steps": int(rn),
                   "note": "device time of neighbour table (build or pair refresh), "
                           "descriptors, networks and forces; the rest of a step is the "
                           "integration kernels and the per-step skin check"},
               "force_rms_eV_per_A": force_rms,
               "fp64_monitor_max_eV_per_atom": max(monitor),
               "energy_drift_max_eV_per_atom": max(drift),
               "timing": "host wall clock around md.run blocks of 10 steps (one sync per "
                         "step for the skin check), FP64 monitor outside",
               "launch_shape": {k: v for k, v in (tuned or {}).items() if k != "all"}}
        md.close()
    finally:
        ann.release()
    return out


def main():
    args = parse()
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()

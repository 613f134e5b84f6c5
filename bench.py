#!/usr/bin/env python
"""Benchmark of the MIS Monte-Carlo Biot-Savart step (particle-steps/s).

Default workload ``tg2048``: Taylor-Green vortex on a periodic unit square,
cell-centred 2048^2 lattice (N = 4,194,304), hwr = 16 (h_w = 1/128),
N1 = N2 = 64 samples per target and sign, dt = 2.5e-4, strengths from the
CG-RBF solve (FP64 dots) of the Taylor-Green field.  Synthetic: no dataset.

GPU arm (default): one step = hash rebuild + MIS velocity of every particle
(both signs) + FP64-wrapped Euler advection, replayed as a CUDA graph.
`value` = N * steps / device time with inputs resident; `e2e` = the same
through the C-ABI host-buffer step (vpmc_sim_step_host: H2D positions, step,
D2H positions + velocities per step).  The working set of a step (candidate
array, 4.3 GB of sample records) is far larger than the 129 MB L2, so no L2
flush is needed between steps.

`--impl reference`: the reference's CPU estimator (monte_carlo_bs_cpu,
restated bit-exactly in oracle/, OpenMP over targets on all host cores) on a
bounded sample of targets of the same workload, one sample per step.

Multi-GPU (torchrun): one job over all ranks (strong scaling).  A single
simulation shards its targets over the ranks, each rank keeping every
particle as a source, and all-gathers the updated positions after each step
(NCCL); an ensemble splits its instances over the ranks with no collective.
value = the job's particles x steps / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at fixed vel. RMS err vs FP64 direct sum; % HBM roofline"

WORKLOADS = {
    "tg2048": dict(Nx=2048, hwr=16.0, N1=64, N2=64, dt=2.5e-4),
    "tg512": dict(Nx=512, hwr=16.0, N1=32, N2=32, dt=5e-4),
    # tg2048's samples per target (and so its queries per bin) on a 512^2 lattice: a
    # profiling-sized stand-in for the bench workload
    "tg512s": dict(Nx=512, hwr=16.0, N1=64, N2=64, dt=5e-4),
    "tg256": dict(Nx=256, hwr=8.0, N1=32, N2=32, dt=1e-3),
    "tg64": dict(Nx=64, hwr=4.0, N1=16, N2=16, dt=1e-3),
    # 64 periodic instances, Nx from {96..384}, 8 Gaussian vortices each, one graph per step
    "ens64": dict(Nx=0, hwr=8.0, N1=32, N2=32, dt=1e-3, ensemble=64),
}

CLOCK_QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines: list[str] = []
        self.th = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={CLOCK_QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.th:
                self.th.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def max_over_ranks(x: float, device=None) -> float:
    """Largest x over the ranks of the default process group (x itself
    without one): the replica timing takes the slowest rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_job: int, steps: int, ms_max: float) -> float:
    """Whole-job units/s: every unit of the job (all ranks together) per step,
    timed by the slowest rank."""
    return units_per_job * steps / (ms_max / 1e3)


def step_flop_rate(sample_queries: float, n_hit: float, ms_per_step: float) -> float:
    """TFLOP/s of a whole step by the algorithmic count: per sample query,
    16 flop per in-support pair plus ~40 flop of MIS arithmetic."""
    return sample_queries * (n_hit * 16.0 + 40.0) / (ms_per_step / 1e3) / 1e12


def reports(rank: int) -> bool:
    """Only rank 0 prints the JSON line (and runs the CPU reference arm)."""
    return rank == 0


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one field-
# evaluation launch, from ncu captures (a constant here: the bench cannot read
# DRAM counters itself).  tg2048: the tg512s capture (same kernel, k_walk,
# queries per thread and queries per bin on a 512^2 lattice, 1/16 of the
# queries) scaled by the 16x queries -- the traffic grows in proportion:
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum --clock-control none
#       -k regex:k_eval -s 1 -c 1 python bench.py --workload tg512s --k 7 --qpt 4 ...
EVAL_DRAM_BYTES_PER_LAUNCH = {
    "tg2048": {"bytes": 16 * 4.248e9, "source": "ncu capture of tg512s (4.248 GB per launch) x 16"},
    "tg512s": {"bytes": 4.248e9, "source": "ncu capture of tg512s"},
}


def eval_traffic(workload: str):
    t = EVAL_DRAM_BYTES_PER_LAUNCH.get(workload)
    return None if t is None else t["bytes"]


def cpu_model() -> str:
    """CPU model name of this host (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


# ------------------------------------------------------------------ CPU side
def in_support_pairs(sim, sps, counts, n_targets=128, seed=5):
    """Mean number of in-support pairs per sample query: over every sample of
    `n_targets` random targets of the last MIS pass's last chunk, the particles
    of the sample's sign subset within h_w of the (wrapped) sample point; a
    sample the unbiased law drops (more than two periods out) or that leaves a
    non-periodic domain counts 0.  Call right after a non-advecting pass, so the
    particles are where the pass drew the samples."""
    from scipy.spatial import cKDTree
    from vortexparticlemc_cuda_gb300.phash import LAW_UNBIASED
    pos_d, om_d, _ = sim.particles()
    pos, om = pos_d.cpu().numpy().astype(np.float64), om_d.cpu().numpy()
    geo = sim.geometry()
    q2 = geo["samples_per_target"]
    t0, _ = sim.read_samples(0, 0)
    nt = geo["N"] - t0
    begins = np.concatenate([[0], np.cumsum(counts)])
    trees = {}
    tot, nq = 0, 0
    for tl in np.random.default_rng(seed).choice(nt, size=min(n_targets, nt), replace=False):
        t = t0 + int(tl)
        i = int(np.searchsorted(begins, t, side="right") - 1)
        sp = sps[i]
        L = np.array([sp.Lx, sp.Ly])
        if i not in trees:
            p, w = pos[begins[i]:begins[i + 1]], om[begins[i]:begins[i + 1]]
            if sp.periodic:
                p = np.mod(p, L)
                p = np.where(p >= L, p - L, p)
            trees[i] = [cKDTree(p[sel], boxsize=L if sp.periodic else None) if sel.any() else None
                        for sel in (w > 0, w < 0)]
        _, y = sim.read_samples(int(tl) * q2, q2)
        y = y.astype(np.float64)
        for sgn in (0, 1):
            ys = y[sgn * (q2 // 2):(sgn + 1) * (q2 // 2)]
            nq += len(ys)
            if sp.periodic:
                k = np.floor(ys / L)
                keep = np.all(np.abs(k) <= 2, 1) if sp.law == LAW_UNBIASED else np.ones(len(ys), bool)
                ys = ys - k * L
                ys = np.where(ys >= L, ys - L, ys)
            else:
                keep = np.all((ys >= 0) & (ys <= L), 1)
            tree = trees[i][sgn]
            if tree is not None and keep.any():
                tot += int(np.sum(tree.query_ball_point(ys[keep], r=sp.h_w, return_length=True)))
    return tot / max(nq, 1)


def cpu_reference_sample(wl, pos, omega, budget_s, seed=17, nthreads=0, fixed_targets=None, st=None):
    """Time the reference CPU estimator (oracle restatement of
    monte_carlo_bs_cpu, pinned bit-exact to the reference sources) on a
    bounded sample of targets.  Returns (particle-steps/s, threads, targets,
    seconds, state); the subsets/hashes (state) are built once, outside the
    timed part."""
    import oracle as O
    prm = O.SimParam(dt=wl["dt"], Nx=wl["Nx"], hwr=wl["hwr"], N1=wl["N1"], N2=wl["N2"])
    if st is None:
        st = O.OracleState(pos, omega, prm)
    rng = np.random.default_rng(seed)
    if fixed_targets is None:
        # a probe large enough to keep every host thread busy sizes the sample
        # to about budget_s seconds
        n_probe = min(len(pos), 512 if nthreads <= 0 else 32 * nthreads)
        t_probe = pos[rng.choice(len(pos), n_probe, replace=False)]
        t0 = time.perf_counter()
        _, nt = O.mc_velocity_omp(st, t_probe, prm.N1, prm.N2, seed, nthreads)
        dt = time.perf_counter() - t0
        m = int(np.clip(n_probe * budget_s / max(dt, 1e-6), 16, 400000))
    else:
        m = fixed_targets
    targets = pos[rng.choice(len(pos), m, replace=m > len(pos))]
    t0 = time.perf_counter()
    vel, nt = O.mc_velocity_omp(st, targets, prm.N1, prm.N2, seed + 1, nthreads)
    _ = targets + np.float32(prm.dt) * vel          # the Euler update of those targets
    dt = time.perf_counter() - t0
    return m / dt, nt, m, dt, st


def cpu_hash_timings(wl, pos, omega, reps=3):
    """The reference's per-step hash rebuild on the host (Simulation::
    do_spatial_hashing: both sign subsets at rsh = Nx / hwr / 2 cells per axis)
    with the oracle's bit-exact restatements: FillCells_cpu + CountingSort_cpu
    (serial, src/cpu/hash.cpp:6-48) and FillCells_omp + CountingSort_omp (all
    host threads, src/omp/hash_omp.cpp:12-70, whose sort output is incorrect).
    Returns ms per rebuild (best of `reps`) and the threads used."""
    import oracle as O
    prm = O.SimParam(dt=wl["dt"], Nx=wl["Nx"], hwr=wl["hwr"])
    s = O.build_subsets(omega)
    px = np.ascontiguousarray(pos[:, 0])
    py = np.ascontiguousarray(pos[:, 1])
    out = {"rsh": prm.rshx, "particles_per_rebuild": int(s["cnt_pos"] + s["cnt_neg"])}
    for kind in ("cpu", "omp"):
        best, nt = 1e30, 1
        for _ in range(reps):
            t0 = time.perf_counter()
            for sub in (s["sub_pos"], s["sub_neg"]):
                if kind == "cpu":
                    cn, ca, vc = O.fill_cells(prm.rshx, prm.rshy, prm.Lx, prm.Ly, sub, px, py)
                    O.counting_sort(cn, ca, vc)
                else:
                    cn, ca, vc, nt = O.fill_cells_omp(prm.rshx, prm.rshy, prm.Lx, prm.Ly, sub, px, py)
                    O.counting_sort_omp(cn, ca, vc)
            best = min(best, time.perf_counter() - t0)
        out[kind] = {"ms_per_rebuild": 1e3 * best, "threads": nt if kind == "omp" else 1,
                     "particles_per_s": out["particles_per_rebuild"] / best}
    out["omp"]["note"] = "CountingSort_omp's output is incorrect (previous-cell base, hash_omp.cpp:65)"
    return out


def strengths_cpu(wl, pos, b):
    """One CG-RBF iteration on the CPU.  On the lattice the Taylor-Green field
    b is an eigenvector of the RBF matrix A, so x0 = b / W(0) and the first CG
    step lands on b / lambda; lambda is read off a few rows of A b (FP64)."""
    import oracle as O
    prm = O.SimParam(dt=wl["dt"], Nx=wl["Nx"], hwr=wl["hwr"], N1=wl["N1"], N2=wl["N2"])
    st = O.OracleState(pos, b, prm)
    rows = np.argsort(-np.abs(b))[:16]
    Ab = O.query_vorticity_f64(st.view("all", w=b), pos[rows], 0, True, False, prm.h_w, True)
    lam = float(np.median(Ab / b[rows].astype(np.float64)))
    return (b.astype(np.float64) / lam).astype(np.float32), dict(iters=1, eigenvalue=lam)


def run_reference(args, wl):
    import oracle as O
    from vortexparticlemc_cuda_gb300 import inputs as In
    rank = int(os.environ.get("RANK", "0"))
    if not reports(rank):
        return 0
    if wl.get("ensemble"):
        # instance 0 of the ensemble; strengths = field x h^2 (the estimator's
        # cost does not depend on the fitted values)
        nxs, p_all, f_all = In.ensemble(wl["ensemble"])
        wl = dict(wl, Nx=nxs[0])
        pos = p_all[: nxs[0] ** 2]
        omega = (f_all[: nxs[0] ** 2] / np.float32(nxs[0] ** 2)).astype(np.float32)
        cg = {"iters": 0, "note": "strengths = field x h^2"}
    else:
        pos = In.lattice(wl["Nx"])
        b = In.taylor_green(pos)
        # one CG iteration: on the lattice the Taylor-Green field is a single
        # Fourier mode of the RBF matrix, so the first step already leaves only
        # FP32 rounding of b; the timed estimator does not depend on the rest
        omega, cg = strengths_cpu(wl, pos, b)
    per_step_budget = (args.ref_seconds if args.ref_seconds > 0
                       else max(1.0, min(20.0, 90.0 / max(1, args.steps + args.warmup))))
    rate, nt, m, dt, st = cpu_reference_sample(wl, pos, omega, per_step_budget)
    N = len(pos)
    # a step of the reference's CPU path: the hash rebuild of both sign subsets
    # (do_spatial_hashing with FillCells_cpu + CountingSort_cpu, all N
    # particles, timed in full) and the estimator + Euler update of every
    # target (timed on m of them, scaled to N)
    times, hash_ms = [], []
    for k in range(args.warmup + args.steps):
        hk = cpu_hash_timings(wl, pos, omega, reps=1)["cpu"]["ms_per_rebuild"]
        r, nt, _, d, _ = cpu_reference_sample(wl, pos, omega, 0, seed=100 + k, fixed_targets=m, st=st)
        if k >= args.warmup:
            times.append(hk / 1e3 + d * N / m)
            hash_ms.append(hk)
    total = sum(times)
    value = N * args.steps / total
    out = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": "synthetic (Taylor-Green lattice)",
        "impl": "reference",
        "config": {"workload": args.workload, **wl, "N": N, "law": "reference CPU (monte_carlo_bs_cpu)",
                   "targets_per_step": m, "hash_rebuild_ms_per_step": float(np.mean(hash_ms)),
                   "step_time": "hash rebuild of all N (both signs, FillCells_cpu + CountingSort_cpu) + the "
                                f"estimator timed on {m} targets and scaled to N"},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": nt, "kind": "port",
                         "cpu_model": cpu_model(),
                         "sample": f"{m} random targets of the {N}-particle workload per step, both signs, "
                                   f"aux=0, Euler update, plus the full hash rebuild; oracle/vpmc_oracle.cpp "
                                   f"restating monte_carlo_bs_cpu and src/cpu/hash.cpp"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cg": cg,
    }
    print(json.dumps(out))
    return 0


# ------------------------------------------------------------------ GPU side
def run_gpu(args, wl):
    import torch
    import torch.distributed as dist

    from vortexparticlemc_cuda_gb300 import inputs as In
    from vortexparticlemc_cuda_gb300 import phash as P

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    law = P.LAW_UNBIASED if args.law == "unbiased" else P.LAW_REFERENCE
    ens = wl.get("ensemble", 0)
    sharded = None
    if ens:
        nxs, pos, field = In.ensemble(ens)
        counts = [nx * nx for nx in nxs]
        n_job = len(pos)
        if world > 1:
            # instances split over ranks by particle count, no collective
            from vortexparticlemc_cuda_gb300.shard import partition_instances
            mine = partition_instances(counts, world)[rank]
            starts = np.concatenate([[0], np.cumsum(counts)])
            pos = np.concatenate([pos[starts[i]:starts[i + 1]] for i in mine])
            field = np.concatenate([field[starts[i]:starts[i + 1]] for i in mine])
            nxs = [nxs[i] for i in mine]
            counts = [counts[i] for i in mine]
            inst_ids = mine
        else:
            inst_ids = list(range(len(nxs)))
        sps = [P.SimParam(dt=wl["dt"], Nx=nx, hwr=wl["hwr"], N1=wl["N1"], N2=wl["N2"], law=law, seed=i)
               for i, nx in zip(inst_ids, nxs)]
    else:
        nxs, pos, field = [wl["Nx"]], In.lattice(wl["Nx"]), None
        counts = [len(pos)]
        n_job = len(pos)
        sps = [P.SimParam(dt=wl["dt"], Nx=wl["Nx"], hwr=wl["hwr"], N1=wl["N1"], N2=wl["N2"], law=law, seed=0)]
    N = len(pos)
    sp = sps[0]
    if world > 1 and not ens:
        # one simulation, targets sharded over the ranks, positions all-gathered after each step
        from vortexparticlemc_cuda_gb300.shard import ShardedSimulation
        sharded = ShardedSimulation(sps, counts, rank, world, device=local)
        sim = sharded.sim
    else:
        sim = P.Simulation(sps, counts)
    step1 = (lambda: sharded.step(1)) if sharded else (lambda: sim.step(1, use_graph=True))  # noqa: E731
    tune = None
    pos_d = torch.from_numpy(pos).to(dev)
    sim.set_particles(pos_d, torch.zeros(N, device=dev))
    log = (lambda m: print(f"[bench {time.strftime('%H:%M:%S')}] {m}", file=sys.stderr, flush=True))  # noqa: E731
    log(f"workload {args.workload}: N={N} in {len(counts)} instance(s), CG init (max {args.cg_iters} iterations)")
    t_cg = time.perf_counter()
    if ens:
        # general right-hand sides on the indefinite RBF matrix: MINRES (CG stalls)
        sim.set_rbf_solver(P.RBF_MINRES)
        infos = sim.init_strengths(torch.from_numpy(field).to(dev), tol=5e-3, max_iter=args.cg_iters)
        cg = {"solver": "minres", "instances": len(infos),
              "max_true_relres": max(i["true_relres"] for i in infos),
              "max_iters": max(i["iters"] for i in infos), "tol": 5e-3,
              "all_at_or_below_tol": all(i["true_relres"] <= 5e-3 for i in infos)}
    else:
        cg = sim.init_strengths(None, tol=1e-8, max_iter=args.cg_iters)[0]
    t_cg = time.perf_counter() - t_cg
    _, omega_d, _ = sim.particles()
    log(f"CG done in {t_cg:.1f} s: {cg}")
    if args.deform:
        # the reference's step_cuda: deformed kernels, 5-point auxiliary targets, F update
        sim.set_deformation(True)
    if args.precision == 64:
        # the plain FP64 GPU path of the same estimator (the comparison baseline of the FP32 path)
        sim.set_precision(64)

    if args.k or args.qpt or args.precision == 64:
        sim.set_tuning(args.k or 4, args.qpt or 4)   # FP64: no autotuning passes (seconds each)
    else:
        t_t = time.perf_counter()
        k_sel, q_sel, best = sim.autotune()
        tune = {"k_walk": k_sel, "queries_per_thread": q_sel, "best_pass_ms": best,
                "seconds": time.perf_counter() - t_t}
        log(f"autotune: {tune}")
    # accuracy at the fixed sample count, with the tuning the timed steps use:
    # velocity RMS error vs the FP64 direct sum at 4096 random particles (seed 2)
    err = None
    if args.err_queries > 0:
        n0 = counts[0]   # instance 0
        idx = np.random.default_rng(2).choice(n0, min(args.err_queries, n0), replace=False)
        v0 = sim.velocity(step=0)
        q = pos_d[torch.from_numpy(idx).to(dev)]
        truth = P.direct_velocity(pos_d[:n0], omega_d[:n0], P.DIRECT_MOLLIFIED, pts=q, param=sp.h_w).cpu().numpy()
        est = v0[torch.from_numpy(idx).to(dev)].cpu().numpy().astype(np.float64)
        rms = np.sqrt(np.mean(np.sum((est - truth) ** 2, 1)))
        ref = np.sqrt(np.mean(np.sum(truth ** 2, 1)))
        err = {"vel_rel_rms_vs_fp64_direct": rms / ref, "queries": int(len(idx))}
        if not ens:
            p = pos[idx].astype(np.float64)
            tg = np.stack([np.sin(2 * np.pi * p[:, 0]) * np.cos(2 * np.pi * p[:, 1]),
                           -np.cos(2 * np.pi * p[:, 0]) * np.sin(2 * np.pi * p[:, 1])], 1)
            err["direct_vs_taylor_green_rel_rms"] = float(np.sqrt(np.mean(np.sum((truth - tg) ** 2, 1))) / ref)
        else:
            err["instance"] = 0

    log(f"accuracy: {err}")
    geo = sim.geometry()
    sim.set_step(0)
    for _ in range(args.warmup):
        step1()
    stream = torch.cuda.current_stream(dev)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    eval_ms = []
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step1()
            eval_ms.append(sim.last_stats()["eval_ms"])
        e1.record(stream)
        torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    log(f"timed {args.steps} steps: {ms / args.steps:.1f} ms/step, eval {np.mean(eval_ms):.1f} ms/step")
    stats = sim.last_stats()
    # in-support pairs per sample query, counted on the samples of one more
    # (non-advecting) pass: the algorithmic work of the evaluation
    sim.velocity()
    n_hit = in_support_pairs(sim, sps, counts)
    log(f"in-support pairs per sample query: {n_hit:.1f}")
    ms = max_over_ranks(ms, dev)
    value = job_throughput(n_job, args.steps, ms)

    # end to end through the host-buffer C-ABI call
    pin = lambda a: torch.from_numpy(a).pin_memory()  # noqa: E731
    hp_in = pin(pos.copy())
    hp_out = pin(np.zeros_like(pos))
    hv_out = pin(np.zeros_like(pos))
    a_in, a_out, a_vel = hp_in.numpy(), hp_out.numpy(), hv_out.numpy()
    d2h = int(2 * pos.nbytes)

    def e2e_step(a_in, a_out, a_vel):
        if sharded is None:
            sim.step_host(a_in, a_out, a_vel)
            return
        # H2D + this rank's shard step, the position all-gather, D2H of all
        # positions and of the shard's velocities
        sim.step_host(a_in, None, None)
        sharded.send_buffer()
        sharded.ex.allgather(sharded.ex.recv, sharded.ex.send)
        sharded.receive()
        torch.from_numpy(a_out).copy_(sharded.full)
        b, e = sharded.ex.begin, sharded.ex.end
        torch.from_numpy(a_vel[b:e]).copy_(sim.particles()[2][b:e])

    if sharded is not None:
        d2h = int(pos.nbytes + 8 * (sharded.ex.end - sharded.ex.begin))
    e2e_step(a_in, a_out, a_vel)        # warm
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_step(a_in, a_out, a_vel)
        a_in, a_out = a_out, a_in
    torch.cuda.synchronize(dev)
    e2e_s = time.perf_counter() - t0
    e2e_ms = max_over_ranks(1e3 * e2e_s, dev)
    e2e = {"value": job_throughput(n_job, args.e2e_steps, e2e_ms), "unit": "particle-steps/s",
           "h2d_bytes_per_step": int(pos.nbytes), "d2h_bytes_per_step": d2h,
           "steps": args.e2e_steps,
           "call": "vpmc_sim_step_host (pinned host buffers)" + (" + position all-gather" if sharded else "")}

    # roofline of the dominant kernel (field evaluation, FP32-pipe bound)
    peaks, peak_kind = measured_peaks()
    Q = 2 * (wl["N1"] + (5 if args.deform else 1) * wl["N2"])
    launches = max(1, geo["chunks"])
    eval_ms_launch = float(np.mean(eval_ms)) / launches
    samples_launch = N * Q / launches
    flop_launch = samples_launch * n_hit * 16.0
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = sm_count * 128 * 2 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    achieved = flop_launch / (eval_ms_launch / 1e3) / 1e12
    clocks = clk.summary()
    roof = {"bound": "fp32", "kernel": ("k_eval, deformed kernels" if args.deform else "k_eval") +
                                       " (field evaluation at MIS samples)",
            "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
            "peak_source": f"{sm_count} SMs x 128 FP32 lanes x 2 x sm_max_mhz from MEASURED_PEAKS.json "
                           f"({peak_kind}); the kernel is FP32-pipe bound: no tensor-core or HBM bound applies",
            "traffic": None if args.deform else eval_traffic(args.workload),
            "traffic_source": None if args.deform else EVAL_DRAM_BYTES_PER_LAUNCH.get(args.workload, {}).get("source"),
            "algorithmic": f"{samples_launch:.0f} sample queries/launch x {n_hit:.1f} in-support pairs x 16 flop",
            "in_support_pairs": ("same-sign particles within h_w of the wrapped sample point (" +
                                 ("isotropic radius, " if args.deform else "") +
                                 "mean over all samples of 128 random targets of a pass; dropped samples count 0)"),
            "eval_ms_per_launch": eval_ms_launch, "eval_share_of_step": float(np.mean(eval_ms)) / (ms / args.steps)}
    if clocks.get("sm_mhz"):
        roof["frac_at_sampled_clock"] = achieved / (sm_count * 128 * 2 * clocks["sm_mhz"] * 1e6 / 1e12)
    # the whole step against the same peak: Q (n_hit 16 + 40) flop per
    # particle-step (16 per in-support pair, ~40 of MIS arithmetic per sample)
    step_achieved = step_flop_rate(samples_launch * launches, n_hit, ms / args.steps)
    roof["step"] = {"achieved": step_achieved, "frac": step_achieved / fp32_peak, "unit": "TFLOP/s",
                    "algorithmic": f"{samples_launch * launches:.0f} sample queries x ({n_hit:.1f} pairs x 16 + 40) "
                                   "flop per step"}

    log(f"e2e {e2e['value']:.3e} particle-steps/s")
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        n0 = counts[0]   # an ensemble's baseline runs on instance 0
        wl0 = dict(wl, Nx=nxs[0])
        om0 = omega_d[:n0].cpu().numpy()
        rate, nt, m, dt, st0 = cpu_reference_sample(wl0, pos[:n0], om0, args.cpu_budget)
        rate1, _, m1, dt1, _ = cpu_reference_sample(wl0, pos[:n0], om0, args.cpu_budget / 2, nthreads=1, st=st0)
        cpu = {"value": rate, "unit": "particle-steps/s", "cores": nt, "kind": "port",
               "sample": f"{m} random targets ({dt:.1f} s), both signs, aux=0, Euler update, reference CPU "
                         f"estimator (monte_carlo_bs_cpu restated in oracle/, bit-exact), OpenMP over targets",
               "value_1_core": rate1, "sample_1_core": f"{m1} random targets ({dt1:.1f} s) on one thread",
               "cpu_model": cpu_model(), "host_threads": os.cpu_count(),
               "hash_rebuild": cpu_hash_timings(wl0, pos[:n0], om0)}
        log(f"CPU baseline: {cpu}")

    out = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f64" if args.precision == 64 else "f32",
        "data": ("synthetic (64 Gaussian-vortex lattices, strengths from CG-RBF)" if ens
                 else "synthetic (Taylor-Green lattice, strengths from CG-RBF)"),
        "config": {"workload": args.workload, **wl, "N": N, "instances": len(counts),
                   **({"Nx_per_instance": nxs} if ens else {}), "law": args.law,
                   "method": "deformation (aux = 1, F update)" if args.deform else "plain", "k_walk": geo["k_walk"],
                   "cells_per_axis": geo["cells_x"], "chunks_per_step": geo["chunks"],
                   "queries_per_thread": sim.tuning()[1],
                   "l2": f"inputs larger than L2 ({N * Q * 16 / 1e9:.1f} GB of sample records + "
                         f"{N * 32 / 1e6:.0f} MB candidates per step)",
                   "parallelism": ("single GPU" if world == 1 else
                                   (f"instances split over {world} ranks (no collective)" if ens else
                                    f"targets sharded over {world} ranks, positions all-gathered per step"))},
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clocks,
        "gpu_launches": int(stats["launches_per_step"] * args.steps),
        "accuracy": err,
        "cg": {**cg, "seconds": t_cg},
        "autotune": tune,
    }
    if reports(rank):
        print(json.dumps(out))
    sim.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="tg2048")
    ap.add_argument("--law", choices=["unbiased", "reference"], default="unbiased")
    ap.add_argument("--k", type=int, default=0, help="walk half-width (0 = auto)")
    ap.add_argument("--qpt", type=int, default=0, help="queries per thread (0 = auto)")
    ap.add_argument("--cg-iters", type=int, default=300)
    ap.add_argument("--err-queries", type=int, default=4096)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ref-seconds", type=float, default=0.0,
                    help="reference arm: CPU seconds of work per step (0: sized so the run takes ~1.5 min)")
    ap.add_argument("--precision", type=int, choices=[32, 64], default=32,
                    help="64: the plain FP64 path (field values, MIS terms, sums in FP64)")
    ap.add_argument("--deform", action="store_true",
                    help="time the deformation step (the reference's step_cuda with aux = 1) instead of the plain one")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gpu":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_gpu(args, wl)


if __name__ == "__main__":
    sys.exit(main())

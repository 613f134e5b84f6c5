#!/usr/bin/env python
"""Accuracy and cost studies of the MIS step beside the throughput bench.

Each study prints one JSON line (stdout) and a short log (stderr).  All FP64
references are the library's own FP64 GPU paths (vpmc_direct_velocity_f64,
vpmc_query_vorticity_f64, the FP64 precision mode of the simulation), which
the `-m gpu` tests pin against the CPU oracle.  Synthetic inputs only.

  --study precision   Taylor-Green, 512^2 lattice, hwr = 16, N1 = N2 = 32, 50
                      steps at dt = 5e-4: FP32-compensated against all-FP64
                      (same estimator, same Philox samples), errors of omega,
                      u and positions at 4096 random particles (seed 1).
  --study inverse     the differentiated inverse problem: 256^2 lattice,
                      hwr = 8, N1 = N2 = 32, 200 steps at dt = 1e-3 with
                      checkpoints every 20; true field = Taylor-Green + 4
                      Gaussian vortices, guess = Taylor-Green; loss = MSE of
                      the final positions against the true run.  Time and
                      device memory of forward + adjoint; the adjoint's
                      gradients along random directions (all strengths
                      scaled by 1 +- 3e-3 z, positions moved by +- 1% of the
                      lattice spacing) against FP64 central differences of
                      the GPU's FP64 forward with the sampling law frozen.
  --study error-cost  2048^2 Taylor-Green, hwr = 16: particle-steps/s and the
                      velocity RMS error against the FP64 direct sum at 4096
                      particles (seed 2) for N1 = N2 in {16, 32, 64, 128, 256},
                      plus the FP64 path's error at N1 = N2 = 64.
  --study variance    the same workload at N1 = N2 = 64: per-particle variance
                      of the unbiased and the reference estimator laws.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def log(msg):
    print(f"[study {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def minimg(d, L=1.0):
    return d - L * np.round(d / L)


def rel_rms(est, truth):
    est, truth = np.asarray(est, np.float64), np.asarray(truth, np.float64)
    return float(np.sqrt(np.mean(np.sum((est - truth).reshape(len(truth), -1) ** 2, 1))) /
                 np.sqrt(np.mean(np.sum(truth.reshape(len(truth), -1) ** 2, 1))))


def make_sim(P, dev, Nx, hwr, N1, N2, dt, law, seed, field=None, solver=None, tol=1e-8, max_iter=5000):
    import torch
    from vortexparticlemc_cuda_gb300 import inputs as In
    pos = In.lattice(Nx)
    sim = P.Simulation(P.SimParam(dt=dt, Nx=Nx, hwr=hwr, N1=N1, N2=N2, law=law, seed=seed), [len(pos)])
    sim.set_particles(torch.from_numpy(pos).to(dev), torch.zeros(len(pos), device=dev))
    if solver is not None:
        sim.set_rbf_solver(solver)
    info = sim.init_strengths(None if field is None else torch.from_numpy(field).to(dev), tol=tol,
                              max_iter=max_iter)[0]
    return sim, pos, info


# ------------------------------------------------------------------ precision
def study_precision(args):
    import torch
    from vortexparticlemc_cuda_gb300 import phash as P
    dev = torch.device("cuda", 0)
    Nx, hwr, N1, N2, dt, T = 512, 16.0, 32, 32, 5e-4, args.steps or 50
    sims, info = {}, None
    for bits in (32, 64):
        sims[bits], pos, info = make_sim(P, dev, Nx, hwr, N1, N2, dt, P.LAW_UNBIASED, seed=1)
        if bits == 64:
            sims[bits].set_precision(64)
        sims[bits].set_tuning(4, 4)
    h_w = P.SimParam(Nx=Nx, hwr=hwr).h_w
    idx = np.random.default_rng(1).choice(len(pos), 4096, replace=False)
    tsel = torch.from_numpy(idx).to(dev)

    def errors(tag):
        out = {}
        p32, om, _ = sims[32].particles()
        p64, om64, _ = sims[64].particles()
        q = p32[tsel]
        # omega: the FP32 query against the FP64 query of the same particles
        w32 = P.query_vorticity(p32, om, q, sign=0, use_signed=True, h_w=h_w).cpu().numpy()
        w64 = P.query_vorticity_f64(p32, om, q, sign=0, use_signed=True, h_w=h_w).cpu().numpy()
        out["omega_rel_rms_fp32_query_vs_fp64"] = rel_rms(w32, w64)
        out["omega_max_err_over_max"] = float(np.abs(w32 - w64).max() / np.abs(w64).max())
        # u: MIS estimate of each path (same step: same samples) vs the FP64 direct sum at its own positions
        for bits, p in ((32, p32), (64, p64)):
            v = sims[bits].velocity(step=10_000)[tsel].cpu().numpy()
            truth = P.direct_velocity(p, om, P.DIRECT_MOLLIFIED, pts=p[tsel], param=h_w).cpu().numpy()
            out[f"u_rel_rms_fp{bits}_vs_fp64_direct"] = rel_rms(v, truth)
            if bits == 32:
                v32 = v
            else:
                out["u_rel_rms_fp32_vs_fp64_path_same_samples"] = rel_rms(v32, v)
        d = minimg(p32.cpu().numpy().astype(np.float64) - p64.cpu().numpy().astype(np.float64))
        out["pos_rms_fp32_vs_fp64"] = float(np.sqrt(np.mean(np.sum(d ** 2, 1))))
        out["pos_max_fp32_vs_fp64"] = float(np.abs(d).max())
        out["pos_rms_over_h"] = out["pos_rms_fp32_vs_fp64"] / (1.0 / Nx)
        log(f"{tag}: {out}")
        return out

    res = {"t0": errors("t=0")}
    for bits in (32, 64):
        sims[bits].set_step(0)
        t0 = time.perf_counter()
        sims[bits].step(T, use_graph=True)
        torch.cuda.synchronize(dev)
        res[f"fp{bits}_seconds_{T}_steps"] = time.perf_counter() - t0
    res[f"t{T}"] = errors(f"t={T} steps")
    out = {"study": "precision", "workload": dict(Nx=Nx, N=len(pos), hwr=hwr, N1=N1, N2=N2, dt=dt, steps=T,
                                                  law="unbiased", seed=1, queries=4096, query_seed=1),
           "cg": info, **res,
           "note": "FP32 = pair arithmetic + compensated MIS sums; FP64 = every pair, term, sum and the Euler "
                   "update in FP64; both draw the same Philox samples; FP64 references are the library's FP64 "
                   "GPU query and direct sum"}
    print(json.dumps(out))


# ------------------------------------------------------------------ inverse
def study_inverse(args):
    import torch
    from vortexparticlemc_cuda_gb300 import inputs as In
    from vortexparticlemc_cuda_gb300 import phash as P
    dev = torch.device("cuda", 0)
    Nx, hwr, N1, N2, dt, T, K = 256, 8.0, 32, 32, 1e-3, args.steps or 200, 20
    seed = 7
    free0 = torch.cuda.mem_get_info(dev)[0]
    pos = In.lattice(Nx)
    field_true = In.inverse_problem_field(pos)
    sim_true, _, info_true = make_sim(P, dev, Nx, hwr, N1, N2, dt, P.LAW_UNBIASED, seed, field=field_true,
                                      solver=P.RBF_MINRES)
    log(f"true field fitted: {info_true}")
    sim_true.set_step(0)
    sim_true.step(T, use_graph=True)
    x_true = sim_true.particles()[0].cpu().numpy().astype(np.float64)
    sim_true.close()

    sim, _, info_guess = make_sim(P, dev, Nx, hwr, N1, N2, dt, P.LAW_UNBIASED, seed)
    _, om_guess, _ = sim.particles()
    om_guess = om_guess.cpu().numpy()
    sim.freeze_sampling(True)
    N = len(pos)
    torch.cuda.synchronize(dev)
    free1 = torch.cuda.mem_get_info(dev)[0]
    sim.set_step(0)
    t0 = time.perf_counter()
    sim.record(T, K)
    torch.cuda.synchronize(dev)
    t_fwd = time.perf_counter() - t0
    free2 = torch.cuda.mem_get_info(dev)[0]
    xt = sim.particles()[0].cpu().numpy().astype(np.float64)
    dX = minimg(xt - x_true)
    loss = float(np.mean(np.sum(dX ** 2, 1)))
    g = torch.from_numpy(2.0 * dX / N).to(dev)
    t0 = time.perf_counter()
    dx0, dw = sim.adjoint(g)
    torch.cuda.synchronize(dev)
    t_adj = time.perf_counter() - t0
    free3 = torch.cuda.mem_get_info(dev)[0]
    dw = dw.cpu().numpy()
    dx0 = dx0.cpu().numpy()
    log(f"loss {loss:.4e}; forward {t_fwd:.2f} s, adjoint {t_adj:.2f} s")

    # the same gradient along the FP64 trajectory
    sim64, _, _ = make_sim(P, dev, Nx, hwr, N1, N2, dt, P.LAW_UNBIASED, seed)
    sim64.set_particles(torch.from_numpy(pos).to(dev), torch.from_numpy(om_guess).to(dev))
    sim64.set_precision(64)
    sim64.set_tuning(4, 4)
    sim64.prepare()
    sim64.freeze_sampling(True)
    sim64.set_step(0)
    t0 = time.perf_counter()
    sim64.record(T, K)
    torch.cuda.synchronize(dev)
    t_fwd64 = time.perf_counter() - t0
    xt64 = sim64.particles()[0].cpu().numpy().astype(np.float64)
    dX64 = minimg(xt64 - x_true)
    loss64 = float(np.mean(np.sum(dX64 ** 2, 1)))
    _, dw64 = sim64.adjoint(torch.from_numpy(2.0 * dX64 / N).to(dev))
    dw64 = dw64.cpu().numpy()
    sim64.close()
    log(f"FP64 trajectory: loss {loss64:.4e}, forward {t_fwd64:.1f} s")

    # FP64 central differences along random directions, one ensemble of
    # 2 x (strength + position directions) instances, all with the guess's
    # seed (so every instance draws the guess run's samples) and the sampling
    # law frozen.  The forward stores positions in FP32 (ulp 6e-8), so a
    # perturbation of one strength by 1e-3 of itself moves positions by less
    # than their resolution; directions over all strengths (and positions)
    # move every particle by many ulps, so the differences resolve the
    # gradient.
    n_dir, n_pdir = args.fd_dirs, args.fd_pos_dirs
    eps_w, eps_x = 3e-3, 1e-2 / Nx                      # relative strength step, position step (1% of h)
    rng = np.random.default_rng(3)
    zs = [rng.choice([-1.0, 1.0], size=N) for _ in range(n_dir)]
    zx = [rng.choice([-1.0, 1.0], size=(N, 2)) for _ in range(n_pdir)]
    nin = 2 * (n_dir + n_pdir)
    sp = P.SimParam(dt=dt, Nx=Nx, hwr=hwr, N1=N1, N2=N2, law=P.LAW_UNBIASED, seed=seed)
    ens = P.Simulation([sp] * nin, [N] * nin)
    ens.set_precision(64)
    ens.set_tuning(4, 4)
    ens.set_particles(torch.from_numpy(np.tile(pos, (nin, 1))).to(dev),
                      torch.from_numpy(np.tile(om_guess, nin)).to(dev))
    ens.prepare()
    ens.freeze_sampling(True)
    om_all, pos_all = [], []
    for z in zs:
        for sgn in (1.0, -1.0):
            w = (om_guess.astype(np.float64) * (1.0 + sgn * eps_w * z)).astype(np.float32)
            om_all.append(w)
            pos_all.append(pos)
    for z in zx:
        for sgn in (1.0, -1.0):
            om_all.append(om_guess)
            pos_all.append((pos.astype(np.float64) + sgn * eps_x * z).astype(np.float32))
    ens.set_particles(torch.from_numpy(np.concatenate(pos_all)).to(dev),
                      torch.from_numpy(np.concatenate(om_all)).to(dev))
    ens.prepare()
    ens.set_step(0)
    t0 = time.perf_counter()
    ens.step(T, use_graph=True)
    torch.cuda.synchronize(dev)
    t_fd = time.perf_counter() - t0
    xa = ens.particles()[0].cpu().numpy().astype(np.float64).reshape(nin, N, 2)
    ens.close()
    losses = np.array([np.mean(np.sum(minimg(xa[i] - x_true) ** 2, 1)) for i in range(nin)])
    rows = []
    for d, z in enumerate(zs):
        # the actual step taken (strengths rounded to FP32), per direction
        wp = om_all[2 * d].astype(np.float64)
        wm = om_all[2 * d + 1].astype(np.float64)
        fd = (losses[2 * d] - losses[2 * d + 1])
        a32 = float(np.dot(dw, wp - wm))
        a64 = float(np.dot(dw64, wp - wm))
        rows.append({"kind": "strengths", "fd": fd, "adjoint_fp32_traj": a32, "adjoint_fp64_traj": a64,
                     "rel_err_fp32": abs(a32 - fd) / abs(fd), "rel_err_fp64": abs(a64 - fd) / abs(fd)})
    for d, z in enumerate(zx):
        i = 2 * (n_dir + d)
        dp = pos_all[i].astype(np.float64) - pos_all[i + 1].astype(np.float64)
        fd = losses[i] - losses[i + 1]
        a32 = float(np.sum(dx0 * dp))
        rows.append({"kind": "positions", "fd": fd, "adjoint_fp32_traj": a32, "rel_err_fp32": abs(a32 - fd) / abs(fd)})
    err_w = max(r["rel_err_fp32"] for r in rows if r["kind"] == "strengths") if n_dir else None
    err_x = max(r["rel_err_fp32"] for r in rows if r["kind"] == "positions") if n_pdir else None
    agree = float(np.linalg.norm(dw - dw64) / np.linalg.norm(dw64))
    log(f"FD ({nin} FP64 forwards, {t_fd:.1f} s): strengths worst {err_w}, positions worst {err_x}; "
        f"FP32 vs FP64 trajectory adjoint {agree:.2e}")
    out = {"study": "inverse",
           "workload": dict(Nx=Nx, N=N, hwr=hwr, N1=N1, N2=N2, dt=dt, steps=T, checkpoint_every=K, law="unbiased",
                            seed=seed, true_field="Taylor-Green + 4 Gaussian vortices (amplitudes N(0,2^2), "
                                                  "radius 0.05, generator seed 7)", guess="Taylor-Green"),
           "fit_true_field_minres": info_true, "fit_guess_cg": info_guess,
           "loss_mse_final_positions": loss, "loss_fp64_trajectory": loss64,
           "forward_record_s": t_fwd, "adjoint_s": t_adj, "forward_record_fp64_s": t_fwd64,
           "device_bytes": {"simulation_and_working_set": int(free0 - free1), "after_record": int(free0 - free2),
                            "after_adjoint": int(free0 - free3)},
           "checkpoints": T // K + 1,
           "fd": {"strength_directions": n_dir, "position_directions": n_pdir, "eps_strength_rel": eps_w,
                  "eps_position": eps_x, "fp64_forwards": nin, "fp64_forward_s": t_fd, "rows": rows,
                  "worst_rel_err_strengths_fp32_traj": err_w, "worst_rel_err_positions_fp32_traj": err_x},
           "dL_domega_fp32_vs_fp64_trajectory": agree,
           "dL_domega_norm": float(np.linalg.norm(dw)),
           "grad_x0_norm": float(np.linalg.norm(dx0)),
           "note": "pathwise adjoint (the discrete CDF choices held: frozen sampling law) with common random "
                   "numbers; finite differences by the GPU's FP64 forward of the same frozen estimator"}
    print(json.dumps(out))


# ------------------------------------------------------------------ error vs cost
def study_error_cost(args):
    import torch
    from vortexparticlemc_cuda_gb300 import phash as P
    dev = torch.device("cuda", 0)
    Nx, hwr, dt = 2048, 16.0, 2.5e-4
    h_w = P.SimParam(Nx=Nx, hwr=hwr).h_w
    idx = np.random.default_rng(2).choice(Nx * Nx, 4096, replace=False)
    tsel = torch.from_numpy(idx).to(dev)
    rows, truth = [], None
    for n in args.samples:
        sim, pos, info = make_sim(P, dev, Nx, hwr, n, n, dt, P.LAW_UNBIASED, seed=0)
        sim.set_tuning(7, 4)
        p, om, _ = sim.particles()
        if truth is None:
            truth = P.direct_velocity(p, om, P.DIRECT_MOLLIFIED, pts=p[tsel], param=h_w).cpu().numpy()
        v = sim.velocity(step=0)[tsel].cpu().numpy()
        err = rel_rms(v, truth)
        fp64 = {}
        if n == 64 and args.fp64:
            # the FP64 path at the same positions and step (same samples)
            sim.set_precision(64)
            sim.set_tuning(4, 4)
            t0 = time.perf_counter()
            v64 = sim.velocity(step=0)[tsel].cpu().numpy()
            fp64 = {"fp64_path_pass_s": time.perf_counter() - t0,
                    "fp64_vel_rel_rms_vs_fp64_direct": rel_rms(v64, truth),
                    "fp32_vs_fp64_path_same_samples": rel_rms(v, v64)}
            sim.set_precision(32)
            sim.set_tuning(7, 4)
        sim.set_step(0)
        sim.step(3, use_graph=True)               # warm-up (graph capture)
        torch.cuda.synchronize(dev)
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        steps = 3
        s.record(torch.cuda.current_stream(dev))
        sim.step(steps, use_graph=True)
        e.record(torch.cuda.current_stream(dev))
        torch.cuda.synchronize(dev)
        ms = s.elapsed_time(e) / steps
        row = {"N1=N2": n, "vel_rel_rms_vs_fp64_direct": err, "ms_per_step": ms,
               "particle_steps_per_s": len(pos) / (ms / 1e3), "eval_ms": sim.last_stats()["eval_ms"], **fp64}
        log(f"{row}")
        rows.append(row)
        sim.close()
    print(json.dumps({"study": "error-cost", "workload": dict(Nx=Nx, N=Nx * Nx, hwr=hwr, dt=dt, law="unbiased",
                                                               k_walk=7, queries_per_thread=4, queries=4096,
                                                               query_seed=2),
                      "rows": rows,
                      "note": "error of one step's velocity (single MC realisation per particle) against the FP64 "
                              "mollified direct sum; it falls as 1/sqrt(samples per target)"}))


# ------------------------------------------------------------------ variance
def study_variance(args):
    """Per-particle variance of the two estimator laws at the bench
    configuration: S velocity passes (S Philox steps) per law, 4096 particles
    (generator seed 2).  The reference law's variance is the figure the
    reference's estimator has (its mean is biased); the unbiased law's is the
    price of its correct mean."""
    import torch
    from vortexparticlemc_cuda_gb300 import phash as P
    dev = torch.device("cuda", 0)
    Nx, hwr, n, dt = 2048, 16.0, 64, 2.5e-4
    S = args.seeds
    sim, pos, info = make_sim(P, dev, Nx, hwr, n, n, dt, P.LAW_UNBIASED, seed=0)
    sim.set_tuning(7, 4)
    p, om, _ = sim.particles()
    h_w = P.SimParam(Nx=Nx, hwr=hwr).h_w
    idx = np.random.default_rng(2).choice(len(pos), 4096, replace=False)
    tsel = torch.from_numpy(idx).to(dev)
    truth = P.direct_velocity(p, om, P.DIRECT_MOLLIFIED, pts=p[tsel], param=h_w).cpu().numpy()
    out = {}
    for name, law in (("unbiased", P.LAW_UNBIASED), ("reference", P.LAW_REFERENCE)):
        sim.set_law(law)
        v = np.stack([sim.velocity(step=5000 + k)[tsel].cpu().numpy() for k in range(S)]).astype(np.float64)
        mean = v.mean(0)
        out[name] = {"per_component_variance": float(v.var(0, ddof=1).mean()),
                     "median_per_particle_variance": float(np.median(v.var(0, ddof=1))),
                     "mean_rel_rms_vs_fp64_direct": rel_rms(mean, truth),
                     "single_estimate_rel_rms_vs_fp64_direct": float(np.mean([rel_rms(v[k], truth) for k in range(S)]))}
        log(f"{name}: {out[name]}")
    out["variance_ratio_unbiased_over_reference"] = (out["unbiased"]["per_component_variance"] /
                                                     out["reference"]["per_component_variance"])
    out["median_variance_ratio"] = (out["unbiased"]["median_per_particle_variance"] /
                                    out["reference"]["median_per_particle_variance"])
    print(json.dumps({"study": "variance", "workload": dict(Nx=Nx, N=len(pos), hwr=hwr, N1=n, N2=n, seeds=S,
                                                             queries=4096, query_seed=2), **out,
                      "note": f"mean of {S} estimates per particle; the reference law's mean is biased "
                              "(its weights do not match its sampling densities)"}))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--study", choices=["precision", "inverse", "error-cost", "variance"], required=True)
    ap.add_argument("--seeds", type=int, default=16, help="variance: estimates per particle and law")
    ap.add_argument("--steps", type=int, default=0, help="steps (0: the study's own count)")
    ap.add_argument("--fd-dirs", type=int, default=4, help="inverse: random strength directions")
    ap.add_argument("--fd-pos-dirs", type=int, default=2, help="inverse: random position directions")
    ap.add_argument("--samples", type=int, nargs="+", default=[16, 32, 64, 128, 256])
    ap.add_argument("--fp64", action="store_true", help="error-cost: also the FP64 path at N1 = N2 = 64")
    args = ap.parse_args()
    {"precision": study_precision, "inverse": study_inverse, "error-cost": study_error_cost,
     "variance": study_variance}[args.study](args)
    return 0


if __name__ == "__main__":
    sys.exit(main())

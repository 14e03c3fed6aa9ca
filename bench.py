#!/usr/bin/env python
"""Benchmark of the mechanical-equilibration path on one GB300.

Workload: 20,000 actin filaments x 50 cylinders (1,000,000 cylinders, 1,020,000
beads) in a 10 um box with 50,000 linkers and 5,000 motors (rest lengths
175-225 nm), seeded synthetic network.  One step = one neighbor-list rebuild
plus one Polak-Ribiere CG minimization from the seeded start until
max|F| < 1 pN (energy-change criterion disabled so that the force criterion
decides), through the C ABI.

Printed line: value = CG force evaluations per second in mixed precision
(force evaluations of the minimizer divided by its time); the time to 1 pN,
the FP64 path's figures and the CPU oracle's are beside it.

--impl reference: the oracle (a loop-for-loop CPU restatement of MEDYAN's
minimizer; MEDYAN itself cannot be built here) on a bounded sample of the
same workload, same metric, on all host threads (OpenMP); the single-thread
figure, MEDYAN's own execution model, is reported beside the GPU line.
"""
from __future__ import annotations

import argparse
import json
import re
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "CG time to 1 pN and force evals/s at 1M cylinders: mixed vs FP64, one GB300"
UNIT = "force_evals/s"
SEED = 20261203 + 2
CONFIG_NAME = "c2"


def profiled_traffic(precision: str):
    """DRAM bytes (read + write) per launch of the mixed trial filament-energy kernel on this
    workload, from the ncu capture summarized in profiles/ (None when absent or FP64)."""
    if precision != "mixed":
        return None
    path = os.path.join(ROOT, "profiles", "k_fil_energy_bulk_trial_1M_cylinders_dram.md")
    try:
        m = re.search(r"dram_bytes_per_launch:\s*(\d+)", open(path).read())
    except OSError:
        return None
    return int(m.group(1)) if m else None

def cg(**kw):
    from picgo_gb300 import cg_params
    base = dict(method=2, max_dist=1.0, lambda_max=0.01, grad_tol=1.0, energy_rel_tol=0.0,
                force_call_limit=1_000_000, energy_call_limit=0)
    base.update(kw)
    return cg_params(**base)


def workload():
    from picgo_gb300 import make_network
    return make_network(CONFIG_NAME, seed=SEED)


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() in ("active", "1"):
                        reasons.add(nm)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def combine_ranks(dist, total_ms: float, force_calls: int, device="cpu"):
    """Whole-job figures over the ranks of a replicas-only run: the slowest
    rank's timed milliseconds and the force evaluations of every rank (one
    replica per rank, no data-path collective).  Identity without a process
    group."""
    if dist is None:
        return total_ms, force_calls
    import torch
    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(force_calls)], dtype=torch.float64, device=device)
    dist.all_reduce(c)
    return float(t.item()), int(round(c.item()))


def flush_l2(torch, dev):
    buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)   # 256 MB > 129 MB L2
    buf.zero_()
    del buf


def run_ours(args, rank, world, dist):
    import numpy as np
    import torch
    from picgo_gb300 import Engine

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    net = workload()
    params = cg()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    eng = Engine(args.precision, local)
    eng.set_network(net)
    if args.graph_mode != "unrolled":
        eng.set_graph_mode(args.graph_mode)
    tuning = eng.autotune()   # launch geometry and bin edge, outside the timed region

    def step():
        eng.reset_coords()
        eng.rebuild()
        return eng.minimize(params)[0]

    for _ in range(args.warmup):
        step()
    # ---- timed: device-resident inputs ----
    results, step_ms, launches = [], [], 0
    with Clocks(local) as clk:
        barrier()
        for _ in range(args.steps):
            flush_l2(torch, dev)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            r = step()
            e1.record()
            torch.cuda.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            results.append(r)
            launches += eng.timing()["launches"]
        barrier()
    clocks = clk.summary()
    force_calls = sum(r["num_force_call"] for r in results)
    total_ms, force_calls_all = combine_ranks(dist, sum(step_ms), force_calls, dev)
    value_local = force_calls / (total_ms / 1e3)
    ms_per_step = total_ms / args.steps

    # ---- end to end: pinned host coordinates in, minimized coordinates out ----
    h_in = torch.empty((net.n_beads, 3), dtype=torch.float64, pin_memory=True)
    h_in.copy_(torch.from_numpy(net.coord))
    h_out = torch.empty((net.n_beads, 3), dtype=torch.float64, pin_memory=True)
    e2e_ms, e2e_calls = [], 0
    barrier()
    for _ in range(args.steps):
        flush_l2(torch, dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.set_coords(h_in.numpy())
        eng.rebuild()
        r = eng.minimize(params)[0]
        h_out.numpy()[:] = eng.coords()
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
        e2e_calls += r["num_force_call"]
    barrier()
    e2e_value = e2e_calls / (sum(e2e_ms) / 1e3)

    # the mixed end state of the last step: coordinates, forces, energy and max |F| as the minimizer reported them
    end_state = {"coord": eng.coords(), "forces": eng.last_forces(), "energy": r["energies_after"][6],
                 "max_force": r["grad_inf_norm"], "iterations": r["num_iter"]}

    # ---- dominant kernel: per-launch device time with CUDA events on the engine's stream ----
    eng.reset_coords()
    eng.rebuild()
    prof = eng.profile(20)
    rs = 4 if args.precision == "mixed" else 8
    nb = prof["n_beads"]
    # Algorithmic bytes per launch (each input read once, each output written once).  The
    # dominant kernel of a minimization is the filament energy of a line-search pass: it
    # reads positions (24 B), flags (1 B), the four per-bead constants and the direction,
    # and writes the trial positions (24 B per trial: the mixed engine evaluates lambda and
    # lambda / 2 in one pass, FP64 one trial).
    trial_writes = 48 if args.precision == "mixed" else 24
    kernels = {
        "fil_energy_trial": (prof["ms_fil_energy_trial"], nb * (24 + 1 + 4 * rs + 3 * rs + trial_writes)),
        "fil_force": (prof["ms_fil_force_kernel"], nb * (24 + 1 + 4 * rs + 3 * rs)),
        "force_gather": (prof["ms_force_gather"],
                         nb * (3 * rs * 3 + 4) + prof["n_slots"] * 3 * rs),
    }
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    name = "fil_energy_trial"
    ms, nbytes = kernels[name]
    achieved = nbytes / (ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": profiled_traffic(args.precision),
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                "bytes_per_launch": int(nbytes), "ms_per_launch": round(ms, 5),
                "others": {k: {"ms": round(v[0], 5), "bytes": int(v[1]),
                               "gbs": round(v[1] / (v[0] * 1e-3) / 1e9, 1)} for k, v in kernels.items() if k != name},
                "profile_ms": {k: round(v, 5) for k, v in prof.items() if k.startswith("ms_")}}
    eng.close()

    out = {
        "metric": METRIC, "value": value_local * world if dist is None else None, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded network generator; no dataset)",
        "config": {"workload": "20,000 filaments x 50 cylinders (1M cylinders), 50k linkers, 5k motors, 10 um box",
                   "seed": SEED, "precision": args.precision, "cg": "Polak-Ribiere, backtracking, gradTol 1 pN, "
                   "maxDist 1, lambdaMax 0.01, energyRelTol 0 (run to 1 pN)",
                   "l2": "flushed (256 MB write) between timed steps", "parallelism": f"replicas x{world}",
                   "graph_mode": args.graph_mode,
                   "tuning": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in tuning.items()}},
        "time_to_1pN_s": round(ms_per_step / 1e3, 4),
        "cg_iterations": results[-1]["num_iter"], "force_calls_per_step": results[-1]["num_force_call"],
        "energy_evals_per_step": results[-1]["num_energy_eval"],
        "line_search_trials_per_step": results[-1]["num_line_search_trials"],
        "final_max_force_pN": results[-1]["grad_inf_norm"],
        "e2e": {"value": round(e2e_value * world, 2), "unit": UNIT, "h2d_bytes_per_step": int(net.n_beads * 24),
                "d2h_bytes_per_step": int(net.n_beads * 24)},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": roofline,
    }
    if dist is not None:
        out["value"] = force_calls_all / (total_ms / 1e3)
    out["value"] = round(out["value"], 2)
    return out, net, end_state


def mixed_end_state_report(net, end, threads: int):
    """The mixed minimizer's end state on the 1M-cylinder network, measured against FP64.

    * same coordinates: the GPU FP64 path and the CPU oracle evaluated at the mixed end
      coordinates with the minimization's own neighbor lists (built once at the start):
      relative energy difference, largest force-component difference, FP64 max |F|;
    * FP64 polish: FP64 CG continued from the mixed end state to the same 1 pN tolerance
      (iterations, relative energy change, bead displacement RMS / max): zero iterations and
      no change when the mixed end state already is an FP64 equilibrium of that tolerance.
    """
    import numpy as np
    import oracle
    from picgo_gb300 import Engine
    x_m, f_m = end["coord"], end["forces"]
    out = {"mixed": {"energy": end["energy"], "max_force_pN": end["max_force"], "iterations": end["iterations"]}}
    with Engine("fp64", int(os.environ.get("LOCAL_RANK", "0"))) as eng:
        eng.set_network(net)
        eng.set_coords(x_m)
        _, e64, _ = eng.energies()
        f64 = eng.forces()
        out["fp64_at_mixed_end"] = {"energy": e64, "energy_rel_diff": abs(end["energy"] - e64) / abs(e64),
                                    "max_force_pN": float(np.abs(f64).max()),
                                    "force_max_abs_diff_pN": float(np.abs(f_m - f64).max())}
        t0 = time.perf_counter()
        r = eng.minimize(cg())[0]
        x_p = eng.coords()
        d = np.linalg.norm(x_p - x_m, axis=1)
        out["fp64_polish_to_1pN"] = {"iterations": r["num_iter"], "seconds": round(time.perf_counter() - t0, 3),
                                     "energy_rel_change": abs(r["energies_after"][6] - e64) / abs(e64),
                                     "max_force_pN": r["grad_inf_norm"],
                                     "displacement_rms_nm": float(np.sqrt((d ** 2).mean())),
                                     "displacement_max_nm": float(d.max())}
    with oracle.threads(threads):
        vec = oracle.vectorize(net)
        e_o = oracle.energy(vec, x_m)
    out["oracle_at_mixed_end"] = {"energy": e_o, "energy_rel_diff": abs(end["energy"] - e_o) / abs(e_o)}
    return out


def fp64_compare(args, net):
    """Same step on the plain FP64 path, once (time to 1 pN and evals/s)."""
    import torch
    from picgo_gb300 import Engine
    eng = Engine("fp64", int(os.environ.get("LOCAL_RANK", "0")))
    eng.set_network(net)
    eng.autotune()
    eng.rebuild()
    r0 = eng.minimize(cg(energy_call_limit=200))[0]   # warm-up
    eng.reset_coords()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.rebuild()
    r = eng.minimize(cg())[0]
    dt = time.perf_counter() - t0
    eng.close()
    return {"time_to_1pN_s": round(dt, 4), "force_evals_per_s": round(r["num_force_call"] / dt, 2),
            "cg_iterations": r["num_iter"], "final_max_force_pN": r["grad_inf_norm"], "status": r["status"],
            "energy_after": r["energies_after"][6], "warmup_iters": r0["num_iter"]}


def c3_report(seed: int = 20261203 + 1):
    """Mixed precision against the FP64 path on the 200 x 20 network (4,000 cylinders, 500 linkers).

    Both minimize from the same seeded start to max|F| < 1 pN; reported: the
    relative energy difference of the end states, their max|F|, the bead
    position RMS / max difference, and the per-evaluation error of the mixed
    engine at the mixed end state (energy relative, force max abs) against FP64
    at the same coordinates.  The FP64 path is the one that matches the CPU
    oracle to 1e-12.
    """
    import numpy as np
    from picgo_gb300 import Engine, make_network
    net = make_network("c1", seed=seed)
    out = {"workload": "200 filaments x 20 cylinders (4,000 cylinders), 500 linkers, 2 um box", "seed": seed}
    ends = {}
    for prec in ("fp64", "mixed"):
        with Engine(prec) as eng:
            eng.set_network(net)
            t0 = time.perf_counter()
            r = eng.minimize(cg(energy_rel_tol=0.0))[0]
            dt = time.perf_counter() - t0
            ends[prec] = (eng.coords(), r)
            out[prec] = {"seconds": round(dt, 4), "cg_iterations": r["num_iter"], "max_force_pN": r["grad_inf_norm"],
                         "energy": r["energies_after"][6], "status": r["status"]}
    (xf, rf), (xm, rm) = ends["fp64"], ends["mixed"]
    d = np.linalg.norm(xm - xf, axis=1)
    out["end_state"] = {"energy_rel_diff": abs(rm["energies_after"][6] - rf["energies_after"][6]) /
                        abs(rf["energies_after"][6]),
                        "max_force_diff_pN": abs(rm["grad_inf_norm"] - rf["grad_inf_norm"]),
                        "position_rms_nm": float(np.sqrt((d ** 2).mean())), "position_max_nm": float(d.max())}
    with Engine("fp64") as e64, Engine("mixed") as emx:
        e64.set_network(net)
        emx.set_network(net)
        e64.set_coords(xm)
        emx.set_coords(xm)
        _, t64, _ = e64.energies()
        _, tmx, _ = emx.energies()
        f64 = e64.forces()
        fmx = emx.forces()
    out["same_coords"] = {"energy_rel_err": abs(tmx - t64) / abs(t64),
                          "force_max_abs_err_pN": float(np.abs(fmx - f64).max()),
                          "force_max_pN": float(np.abs(f64).max())}
    return out


def c5_report(n_params: int = 64, seed: int = 20261203 + 5, budget_s: float = 240.0):
    """Implicit adjoint on the 2,000 x 30 network with 5,000 linkers (k ~ U(4, 12),
    l0 ~ U(20, 40)): L = E(x*) + mean over filaments |end - start|^2.  The adjoint
    gradient of L in per-linker k and l0 (GPU FP64: CG, Newton refinement to 1e-9 pN,
    one Hessian CG solve) against central differences (h = 1e-4 relative) of the FP64
    reference on `n_params` random parameters: each side re-equilibrated from x* by
    Newton refinement alone (x*(theta +- h) is a 1e-4 perturbation of x*), its loss
    evaluated by the CPU oracle at the refined coordinates with the device's lists.
    The lists stay those the FP64 minimization was run with (built at its start):
    E is the energy of that fixed list, as in one MEDYAN minimization, and a list
    rebuilt at x* after the long descent would hold pairs that moved into contact
    while no term kept them apart.  Parameters are checked until `budget_s` seconds
    of finite differences have passed; the report says how many were."""
    import numpy as np
    import oracle
    from picgo_gb300 import Engine, make_network
    net = make_network("c5", seed=seed)
    fcs = np.asarray(net.fil_cyl_start)
    first, last = net.cyl_b1[fcs[:-1]], net.cyl_b2[fcs[1:] - 1]

    def reg(x):
        d = x[last] - x[first]
        g = np.zeros_like(x)
        np.add.at(g, last, 2.0 * d / len(first))
        np.add.at(g, first, -2.0 * d / len(first))
        return float((d * d).sum(1).mean()), g

    k0 = np.asarray(net.lk_k, dtype=np.float64)
    l00 = np.asarray(net.lk_l0, dtype=np.float64)
    out = {"workload": "2,000 filaments x 30 cylinders (60,000 cylinders), 5,000 linkers k~U(4,12) l0~U(20,40)",
           "seed": seed, "n_params": n_params}
    def log(msg):
        print(f"c5 [{time.perf_counter() - t0:7.1f} s] {msg}", file=sys.stderr, flush=True)

    t0 = time.perf_counter()
    with Engine("mixed") as em:   # most of the descent in mixed precision, to its 1 pN design point
        em.set_network(net)
        r = em.minimize(cg())[0]
        x0 = em.coords()
    log(f"mixed CG to 1 pN: {r['num_iter']} iterations")
    with Engine("fp64") as eng:
        eng.set_network(net)
        eng.set_coords(x0)
        eng.rebuild()   # the lists of this minimization, at x0; kept through Newton, adjoint and FD
        x_lists = x0
        # FP64 CG to 1e-2 pN, then damped Newton; where Newton meets negative
        # curvature the CG end was not a strict minimum (it descends from
        # there), so CG and Newton alternate until Newton converges on a
        # positive-definite Hessian or the equilibration budget runs out
        stages = []
        for stage in range(8):
            r = eng.minimize(cg(grad_tol=1e-2, force_call_limit=400_000))[0]
            info = eng.newton_refine(40, 1e-9, 1e-8, 20000)
            stages.append({"cg_iterations": r["num_iter"], "cg_max_force_pN": r["grad_inf_norm"],
                           "newton_steps": info["newton_steps"], "newton_cg_iterations": info["iterations"],
                           "newton_max_force_pN": info["max_force"],
                           "negative_curvature": info["negative_curvature"]})
            log(f"stage {stage}: FP64 CG {r['num_iter']} iterations to {r['grad_inf_norm']:.3g} pN; Newton "
                f"{info['newton_steps']} steps, {info['iterations']} CG iterations, max|F| {info['max_force']:.3g}, "
                f"negative curvature {info['negative_curvature']}")
            if info["max_force"] < 1e-6 and not info["negative_curvature"]:
                break
            if time.perf_counter() - t0 > 0.6 * budget_s:
                break
        xs = eng.coords()
        out["equilibration_stages"] = stages
        out["equilibrate_s"] = round(time.perf_counter() - t0, 2)
        out["equilibrium_max_force_pN"] = info["max_force"]
        out["strict_minimum"] = bool(info["max_force"] < 1e-6 and not info["negative_curvature"])
        lx, g = reg(xs)
        ta = time.perf_counter()
        gk, gl, ainfo = eng.adjoint(g, 1.0)
        out["adjoint_s"] = round(time.perf_counter() - ta, 3)
        out["adjoint_cg"] = {k: ainfo[k] for k in ("iterations", "converged", "rel_residual")}
        rng = np.random.default_rng(seed)
        picks = rng.choice(len(k0), size=max(1, n_params // 2), replace=False)
        rows, worst, t_fd = [], 0.0, time.perf_counter()
        log(f"adjoint: {out['adjoint_s']} s, {ainfo['iterations']} CG iterations")
        for j in picks:
            if time.perf_counter() - t_fd > budget_s:
                break
            for which in ("k", "l0"):
                base = k0 if which == "k" else l00
                h = 1e-4 * base[j]
                vals = []
                for sgn in (1, -1):
                    p = base.copy()
                    p[j] += sgn * h
                    kk, ll = (p, l00) if which == "k" else (k0, p)
                    eng.set_coords(xs)
                    eng.set_linker_params(kk, ll)
                    ninfo = eng.newton_refine(8, 1e-9, 1e-8, 20000)
                    xe = eng.coords()
                    side = net.copy()
                    side.lk_k, side.lk_l0 = kk, ll
                    vec = oracle.vectorize(side, x_lists)   # the device's lists
                    vals.append(oracle.energy(vec, xe) + reg(xe)[0])
                fd = (vals[0] - vals[1]) / (2 * h)
                adj = float((gk if which == "k" else gl)[j])
                rel = abs(adj - fd) / max(abs(fd), 1e-12)
                worst = max(worst, rel)
                rows.append({"param": f"{which}[{int(j)}]", "adjoint": adj, "fd": fd, "rel_err": rel,
                             "newton_max_force_pN": ninfo["max_force"], "newton_steps": ninfo["newton_steps"],
                             "newton_cg_iterations": ninfo["iterations"]})
                log(f"{which}[{int(j)}] rel {rel:.2e}")
        eng.set_linker_params(k0, l00)
        out["fd_s"] = round(time.perf_counter() - t_fd, 2)
        out["n_checked"] = len(rows)
        out["checks"] = rows
        out["max_rel_err"] = worst
    return out


def c4_report(n_replicas: int, precision: str = "mixed", loop_budget_s: float = 240.0):
    """Batched ensemble: `n_replicas` independent networks of uneven size
    (filaments log-uniform on 50-5,000, 20-50 cylinders each, C1 density)
    minimized together in one context vs one after another; replicas/s.  The
    one-after-another loop runs over a seeded random order of the replicas until
    `loop_budget_s` seconds have passed; its replicas/s is that sample's rate
    (cylinder-weighted extrapolation beside it)."""
    import torch
    from picgo_gb300 import Engine
    from picgo_gb300.network import make_ensemble
    t0 = time.perf_counter()
    nets = make_ensemble(n_replicas)
    t_gen = time.perf_counter() - t0
    ncyl = sum(n.n_cyl for n in nets)
    prm = cg(energy_rel_tol=0.0)
    out = {"workload": f"{n_replicas} replicas, filaments log-uniform 50-5,000, 20-50 cylinders, C1 density",
           "n_replicas": n_replicas, "cylinders_total": ncyl, "precision": precision,
           "generate_s": round(t_gen, 1)}
    with Engine(precision) as eng:
        eng.set_networks(nets)
        eng.minimize(cg(energy_call_limit=20))           # warm-up: graph capture, first launches
        eng.reset_coords()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.rebuild()
        res = eng.minimize(prm)
        t_b = time.perf_counter() - t0
    out["batched"] = {"seconds": round(t_b, 3), "replicas_per_s": round(n_replicas / t_b, 2),
                      "converged": sum(1 for r in res if r["status"] == 0 and r["grad_inf_norm"] < 1.0),
                      "max_iterations": max(r["num_iter"] for r in res)}
    print(f"c4: batched {t_b:.1f} s", file=sys.stderr, flush=True)
    import numpy as np
    order = np.random.default_rng(20261203).permutation(n_replicas)
    t_loop, conv, done, cyl_done = 0.0, 0, 0, 0
    with Engine(precision) as eng:
        for i in order:
            if t_loop > loop_budget_s:
                break
            net = nets[int(i)]
            eng.set_network(net)
            if done == 0:
                eng.minimize(cg(energy_call_limit=20))
                eng.reset_coords()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            eng.rebuild()
            r = eng.minimize(prm)[0]
            t_loop += time.perf_counter() - t0
            conv += int(r["status"] == 0 and r["grad_inf_norm"] < 1.0)
            done += 1
            cyl_done += net.n_cyl
    rate = done / t_loop
    out["looped"] = {"replicas_run": done, "seconds": round(t_loop, 3), "replicas_per_s": round(rate, 3),
                     "converged": conv, "cylinders_run": cyl_done,
                     "extrapolated_seconds_all": round(t_loop * ncyl / max(cyl_done, 1), 1)}
    out["batched_vs_looped"] = round((n_replicas / t_b) / rate, 3)
    return out


def cpu_sample(net, seconds: float, threads: int = 1):
    """The oracle's CG on the same network, bounded: force evaluations per second
    on `threads` host threads (1 = serial, like MEDYAN's minimizer)."""
    import oracle
    t0 = time.perf_counter()
    vec = oracle.vectorize(net)
    t_vec = time.perf_counter() - t0
    limit = 8
    with oracle.threads(threads):
        while True:
            t0 = time.perf_counter()
            x, f, res = oracle.minimize(vec, net.coord, oracle.cg_params(energyRelTol=0.0, energyCallLimit=limit,
                                                                           forceCallLimit=1_000_000))
            dt = time.perf_counter() - t0
            if dt >= seconds or limit >= 4096:
                break
            limit = int(limit * max(2.0, min(8.0, seconds / max(dt, 1e-3))))
    how = "single-threaded like MEDYAN's minimizer" if threads == 1 else \
        f"OpenMP over {threads} host threads (force fields and CG vector loops)"
    return {"value": round(res.numForceCall / dt, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"oracle CG on the same 1M-cylinder network from the same start, first {res.numIter} "
                      f"iterations ({res.numForceCall} force + {res.numEnergyCall} energy evaluations) in {dt:.1f} s "
                      f"(vectorize {t_vec:.1f} s excluded); {how}; host {platform.machine()}, "
                      f"{os.cpu_count()} logical CPUs",
            "seconds": round(dt, 2), "energy_evals_per_force_eval": round(res.numEnergyCall / max(1, res.numForceCall), 3)}


def cpu_time_to_1pN(net, threads: int):
    """The oracle's CG from the seeded start to max|F| < 1 pN, unbounded (wall time)."""
    import oracle
    vec = oracle.vectorize(net)
    with oracle.threads(threads):
        t0 = time.perf_counter()
        x, f, res = oracle.minimize(vec, net.coord, oracle.cg_params(energyRelTol=0.0, forceCallLimit=10_000_000))
        dt = time.perf_counter() - t0
    return {"time_to_1pN_s": round(dt, 2), "cores": threads, "cg_iterations": res.numIter,
            "force_calls": res.numForceCall, "energy_calls": res.numEnergyCall, "final_max_force_pN": res.gradInfNorm,
            "force_evals_per_s": round(res.numForceCall / dt, 3)}


def host_threads() -> int:
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except (AttributeError, OSError):
        return max(1, os.cpu_count() or 1)


def run_reference(args, rank, world):
    if rank != 0:
        return None
    net = workload()
    vals = []
    for _ in range(args.warmup):
        pass   # the oracle has no warm-up state; each step is a fresh bounded sample
    for _ in range(args.steps):
        s = cpu_sample(net, args.cpu_seconds / max(1, args.steps), host_threads())
        vals.append(s)
    v = sum(s["value"] for s in vals) / len(vals)
    cpu = dict(vals[-1])
    cpu["value"] = round(v, 4)
    return {"metric": METRIC, "value": round(v, 4), "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded network generator; no dataset)",
            "config": {"workload": "20,000 filaments x 50 cylinders (1M cylinders), 50k linkers, 5k motors, 10 um box",
                       "seed": SEED, "precision": "fp64 (CPU restatement of MEDYAN's minimizer, all host threads)"},
            "cpu_baseline": cpu,
            "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def probe(args):
    """A bounded piece of the minimization for profiler captures and quick timings.

    Default: neighbor-list rebuild + Polak-Ribiere CG from the seeded start until
    `--energy-calls` energy calls (every kernel of real CG iterations);
    `--evals N`: each evaluation kernel launched N times through mech_profile;
    `--forces N` / `--energies N`: only that many mech_forces / mech_energy calls,
    so that a profiler's first matching launches are those of one evaluation kind.
    Prints one JSON line.
    """
    from picgo_gb300 import Engine, make_network
    net = make_network(args.workload, seed=args.seed)
    out = {"probe": args.workload, "precision": args.precision, "n_beads": net.n_beads}
    with Engine(args.precision) as eng:
        eng.set_network(net)
        if args.autotune:
            out["tuning"] = eng.autotune()
        out["lists"] = eng.rebuild()
        if args.forces > 0 or args.energies > 0:
            for _ in range(args.forces):
                eng.forces()
            for _ in range(args.energies):
                eng.energies()
            out["calls"] = {"forces": args.forces, "energies": args.energies}
        elif args.evals > 0:
            out["profile"] = eng.profile(args.evals)
        else:
            if args.skip_calls > 0:
                # descend first without a timeline (a diagnostic build writes one
                # per minimization when MECH_TRACE_FILE is set)
                dump = os.environ.pop("MECH_TRACE_FILE", None)
                eng.minimize(cg(energy_call_limit=args.skip_calls))
                if dump is not None:
                    os.environ["MECH_TRACE_FILE"] = dump
            t0 = time.perf_counter()
            r = eng.minimize(cg(energy_call_limit=args.energy_calls))[0]
            out["seconds"] = round(time.perf_counter() - t0, 4)
            out.update({k: r[k] for k in ("num_iter", "num_force_call", "num_energy_eval", "grad_inf_norm",
                                          "status")})
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--graph-mode", default="unrolled", choices=["unrolled", "unrolled_pdl", "unrolled_coop", "conditional"],
                    help="how the minimizer drives the device (the mixed run; the FP64 comparison keeps the default)")
    ap.add_argument("--cpu-full", action="store_true",
                    help="also run the oracle's CG to 1 pN unbounded: the 200 x 20 network serially and on all host "
                         "threads, and this workload on all host threads (minutes)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-c3", action="store_true", help="skip the mixed-vs-FP64 end-state report on the small network")
    ap.add_argument("--c5", type=int, default=0, metavar="P",
                    help="only run the implicit-adjoint check on P parameters of the 2,000 x 30 network (64 in the "
                         "configuration)")
    ap.add_argument("--c4", type=int, default=0, metavar="R",
                    help="only run the batched-ensemble comparison on R replicas and print its JSON line")
    ap.add_argument("--probe", action="store_true",
                    help="profiler probe: a bounded minimization (or single evaluations) of --workload, one JSON line")
    ap.add_argument("--workload", default="c2", help="probe: network config name (c1, c2, c5)")
    ap.add_argument("--seed", type=int, default=None, help="probe: network seed (default: the config's)")
    ap.add_argument("--energy-calls", type=int, default=40, help="probe: energy calls of the bounded minimization")
    ap.add_argument("--skip-calls", type=int, default=0,
                    help="probe: energy calls of an earlier minimization from the start, without a timeline")
    ap.add_argument("--evals", type=int, default=0, help="probe: launches per evaluation kernel (mech_profile)")
    ap.add_argument("--forces", type=int, default=0, help="probe: only this many mech_forces calls")
    ap.add_argument("--energies", type=int, default=0, help="probe: only this many mech_energy calls")
    ap.add_argument("--autotune", action="store_true", help="probe: run the autotuner first")
    args = ap.parse_args()
    if args.probe:
        probe(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl" if args.impl == "ours" else "gloo")
        dist = tdist
    if args.c5 > 0:
        if rank == 0:
            print(json.dumps({"c5": c5_report(args.c5)}))
        return
    if args.c4 > 0:
        if rank == 0:
            print(json.dumps({"c4": c4_report(args.c4, args.precision)}))
        return
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out))
        if dist is not None:
            dist.destroy_process_group()
        return
    out, net, end = run_ours(args, rank, world, dist)
    if rank == 0:
        if not args.no_fp64 and args.precision == "mixed":
            f = fp64_compare(args, net)
            out["fp64"] = f
            out["mixed_vs_fp64_time_to_1pN"] = round(f["time_to_1pN_s"] / out["time_to_1pN_s"], 3)
            out["mixed_vs_fp64_evals_per_s"] = round(out["value"] / max(f["force_evals_per_s"], 1e-9), 3)
            out["mixed_vs_fp64_us_per_iteration"] = round(
                (f["time_to_1pN_s"] / f["cg_iterations"]) / (out["time_to_1pN_s"] / out["cg_iterations"]), 3)
            out["mixed_end_state"] = mixed_end_state_report(net, end, host_threads())
        if not args.no_c3:
            out["c3_mixed_vs_fp64"] = c3_report()
        if not args.no_cpu and world == 1:
            out["cpu_baseline"] = cpu_sample(net, args.cpu_seconds * 0.6, host_threads())
            one = cpu_sample(net, args.cpu_seconds * 0.4, 1)
            out["cpu_baseline_1thread"] = {k: one[k] for k in ("value", "unit", "cores", "seconds")}
            if args.cpu_full:
                from picgo_gb300 import make_network
                out["cpu_baseline"]["time_to_1pN"] = cpu_time_to_1pN(net, host_threads())
                c1 = make_network("c1", seed=20261203 + 1)
                out["cpu_c1_time_to_1pN"] = {"threads": cpu_time_to_1pN(c1, host_threads()),
                                             "serial": cpu_time_to_1pN(c1, 1)}
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

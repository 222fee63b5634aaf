#!/usr/bin/env python
"""Throughput of the particle-field step on GB300.

Workload: 256^3 grid (box 256, spacing 1) + 64 semiflexible chains x 500
beads = 32,000 beads, kT = 1, dt = 1e-4 (synthetic, seeded; no dataset).
A "step" is one full timestep of the hot path: neighbor check/rebuild,
lj/cut + gridatom/gaussian pair forces and mu deposit, chain integration,
Flory-Huggins mu, r2c(mu), Model-B update with conserved noise, c2r to phi
and grad phi.  Grid arithmetic FP32, bead positions FP64.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

N > 1 runs under torchrun: every rank advances an independent replica (its
own seeds) on its own GPU with no data-path collective ("replicas only");
value = steps of all ranks / max-over-ranks time.

--impl reference times the reference's CPU algorithm (the FP64 oracle
restatement: the reference itself cannot be built here) on the same
workload on every host core, rank 0 only.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "steps/s at 256^3 grid+32k beads, fraction of HBM roofline; learned vs plain"
WORKLOAD = "256cube_32kbeads"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default=WORKLOAD)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-learned", action="store_true", help="skip the learned-vs-plain part of the default line")
    p.add_argument("--no-fp64", action="store_true", help="skip the FP64 throughput figure")
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the default kernel variants (profiling runs: timings under a profiler mislead the tuner)")
    p.add_argument("--profile-steps", type=int, default=5)
    p.add_argument("--traj", type=int, default=48, help="training trajectories of the learned workloads")
    p.add_argument("--epochs", type=int, default=6, help="training epochs of the learned workloads")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = []
        smax = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_model():
    """The host CPU's model name (lscpu; /proc/cpuinfo as fallback)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def stage_bytes(cfg, s):
    """Compulsory HBM bytes of each stage of the resident step, per step.
    N real nodes, Nc complex modes, s bytes per real (4 in FP32)."""
    n = cfg["n"]
    N = n ** 3
    Nc = (n // 2 + 1) * n * n
    return {
        "x_r2c_fh": 2 * s * N + 2 * s * Nc,   # read phi, deposit; write x-transformed mu
        "y_fft": 4 * s * Nc,                  # read + write one spectrum
        "z_update_ifft": 10 * s * Nc,         # read mu (x,y done), phi_hat; write phi_hat', A, B
        "y_ifft": 10 * s * Nc,                # read A, B; write C, D, E
        "x_c2r": 6 * s * Nc + 4 * s * N,     # read C, D, E; write phi, dphi/dx, dphi/dy, dphi/dz
    }


def ncu_traffic():
    """DRAM bytes per step of each stage from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "ncu_dram_bytes_256cube.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            parts = line.split()
            if len(parts) == 2 and not line.startswith("#"):
                try:
                    out[parts[0]] = float(parts[1])
                except ValueError:
                    pass
    return out


def make_chains(cfg, rank):
    from phafd_gb300 import workloads as W
    return W.random_walk_chains(cfg["nchains"], cfg["chain_len"], cfg["origin"], cfg["L"],
                                cfg["chain_seed"] + 1000 * rank, cfg["bond"])


def replica_cfg(cfg, rank):
    """Rank r advances an independent replica: the same workload with its own seeds."""
    c = dict(cfg)
    c["grid_seed"] = cfg["grid_seed"] + 1000 * rank
    c["chain_seed"] = cfg["chain_seed"] + 1000 * rank
    return c


def max_over_ranks(value, dist=None, device=None):
    """The slowest rank's time (all_reduce MAX); the value itself at N = 1."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, steps, ms_max):
    """Whole-job steps/s: every rank advanced `steps` steps of its own replica."""
    return world * steps / (ms_max / 1000.0)


def cpu_baseline_oracle(cfg, chains, nsteps):
    """The reference's algorithm (FP64 oracle restatement) on every host core
    the process may use, on a bounded sample of the workload: set-up untimed,
    then `nsteps` steps.  Returns (steps/s, seconds, threads)."""
    from oracle import oracle as OR
    from oracle.oracle import Oracle
    from phafd_gb300 import workloads as W
    threads = OR.host_threads()
    OR.set_threads(threads)
    o = Oracle()
    W.apply(o, cfg, chains=chains)
    o.setup()
    t0 = time.perf_counter()
    o.run(nsteps)
    dt = time.perf_counter() - t0
    return nsteps / dt, dt, threads


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from phafd_gb300 import workloads as W
    from oracle import build as OB
    OB.build()
    cfg = replica_cfg(W.CONFIGS[args.workload], 0)
    chains = make_chains(cfg, 0)
    timed = max(1, min(args.steps, 3))
    warm = 1 if args.warmup > 0 else 0
    from oracle import oracle as OR
    from oracle.oracle import Oracle
    threads = OR.host_threads()
    OR.set_threads(threads)
    o = Oracle()
    W.apply(o, cfg, chains=chains)
    o.setup()
    if warm:
        o.run(warm)
    t0 = time.perf_counter()
    o.run(timed)
    dt = time.perf_counter() - t0
    v = timed / dt
    sample = ("%d timed steps of %s after set-up and %d warm-up step(s); FP64 oracle restatement of the "
              "reference's CPU path, grid loops (FFT lines, pointwise passes, mode update) on %d threads, "
              "bead loops on one" % (timed, args.workload, warm, threads))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": timed, "warmup": warm, "ms_per_step": 1000.0 * dt / timed, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "grid": [cfg["n"]] * 3, "beads": W.nbeads(cfg),
                   "parallelism": "1 process, %d threads" % threads},
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    rank, world, local = dist_env()
    import numpy as np
    from phafd_gb300 import build as B
    B.build()
    from phafd_gb300 import workloads as W
    from phafd_gb300.gpu import PhafdGPU

    torch_dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        torch_dist = dist

    def barrier():
        if torch_dist:
            torch_dist.barrier()

    def ranks_max(v):
        return max_over_ranks(v, torch_dist, "cuda")

    cfg = replica_cfg(W.CONFIGS[args.workload], rank)
    chains = make_chains(cfg, rank)

    def device_free():
        try:
            import torch
            return torch.cuda.mem_get_info(local)
        except Exception:  # no torch: the footprint is not reported
            return None, None

    free0, total = device_free()
    g = PhafdGPU(precision=32, device=local, schedule="resident")
    W.apply(g, cfg, chains=chains)
    g.setup()
    g.run(1)
    free1, _ = device_free()
    memory = None if free0 is None else {"context_bytes": int(free0 - free1), "device_total_bytes": int(total),
                                         "note": "device memory taken by the context (state, lists, spectra, "
                                                 "graphs) after set-up and one step: free before minus free after"}
    # clocks are sampled from the warm-up through the timed region and a
    # continuation of the same steps of at least one second
    sampler = ClockSampler(local)
    sampler.start()
    g.run(max(args.warmup, 3))
    # the project's autotuner picks the kernel variants on the run's own steps
    best, tune_ms = g.autotune(10) if not args.no_autotune else (12, np.zeros(16))
    names = {0: "register-resident 256, x passes loading their own tiles", 1: "plane-fused x/y", 2: "generic 256 tiles",
             3: "plane-fused x/y + generic 256 tiles", 4: "register-resident 256, tensor-map fed x c2r",
             8: "register-resident 256, tensor-map fed x r2c",
             12: "register-resident 256, tensor-map fed x r2c and x c2r (default)"}
    autotune = {"best": names[best], "ms_per_step": {names[f]: (float(tune_ms[f]) if tune_ms[f] > 0 else None)
                                                      for f in names}}

    # stage profile (eager steps with events between stages; not the timed region)
    prof = g.profile_stages(args.profile_steps)
    g.run(2)

    barrier()
    g.synchronize()
    ms = g.run_timed(args.steps)
    g.synchronize()
    barrier()
    ms_max = ranks_max(ms)
    t_soak = time.perf_counter()
    while time.perf_counter() - t_soak < 1.0:
        g.run(200)
        g.synchronize()
    clocks = sampler.stop()
    clocks["window"] = "warm-up, timed region and 1 s more of the same steps (50 ms sampling)"
    counters = g.counters()

    value = job_throughput(world, args.steps, ms_max)
    peak, peak_kind = measured_peak()
    s = 4
    sb = stage_bytes(cfg, s)
    grid_stages = {k: prof[k] for k in sb}
    dom = max(grid_stages, key=grid_stages.get)
    achieved = sb[dom] / (prof[dom] / 1000.0) / 1e9
    traffic = ncu_traffic().get(dom)
    bstep = W.algorithmic_bytes_per_step(cfg, s)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of this stage in one ncu capture "
                                  "(profiles/ncu_dram_bytes_256cube.txt), not measured in this run",
                "algorithmic_bytes_per_launch": sb[dom], "launch_ms": prof[dom]}
    step_roofline = {"bytes_per_step": bstep, "achieved": bstep / (ms_max / args.steps / 1000.0) / 1e9,
                     "peak": peak, "unit": "GB/s"}
    step_roofline["frac"] = step_roofline["achieved"] / peak

    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "grid": [cfg["n"]] * 3, "beads": W.nbeads(cfg),
                   "schedule": "resident", "bead_positions": "f64",
                   "parallelism": "replicas x%d" % world,
                   "l2": "working set ~0.9 GB > 129 MB L2 (no flush needed)"},
        "roofline": roofline,
        "step_roofline": step_roofline,
        "stage_ms": prof,
        "autotune": autotune,
        "memory": memory,
        "clocks": clocks,
        "gpu_launches": int(counters.get("kernels_per_step", 0)) * args.steps if counters.get("kernels_per_step") else None,
        "neighbor_calls": counters["neighbor_calls"],
    }
    phi_host = np.ascontiguousarray(g.grid_get("phi"))
    g.close()

    # the same workload through the FP64 path (the precision the reference computes in)
    if not args.no_fp64:
        g64 = PhafdGPU(precision=64, device=local, schedule="resident")
        W.apply(g64, cfg, chains=chains)
        g64.setup()
        g64.run(max(args.warmup, 3))
        k64 = max(20, min(args.steps, 200))
        barrier()
        ms64 = ranks_max(g64.run_timed(k64))
        line["fp64"] = {"value": job_throughput(world, k64, ms64), "unit": "steps/s", "steps": k64,
                        "ms_per_step": ms64 / k64,
                        "step_roofline_frac": W.algorithmic_bytes_per_step(cfg, 8) / (ms64 / k64 / 1000.0) / 1e9 / peak}
        g64.close()

    # end to end through the public C ABI with host buffers: set-up (context,
    # upload of the state from host memory, lists, graph) timed apart from the
    # steady steps; every step's bead result (x, ux, F, image flags) lands in
    # page-locked host memory, read back pipelined with the steps (step s + 1
    # is enqueued before the host waits for step s's copy), and the same with
    # a blocking read after each step for comparison
    if not args.no_e2e:
        from phafd_gb300 import gpu as G
        k = max(20, min(args.steps, 200))
        xs = chains[0]
        nb = W.nbeads(cfg)
        t0 = time.perf_counter()
        e = PhafdGPU(precision=32, device=local, schedule="resident")
        W.apply(e, cfg, chains=chains, phi=phi_host)  # the state from host arrays: phi, then the beads
        e.setup()
        e.run(1)
        e.atoms_get()
        bufs = [(np.empty((nb, 3)), np.empty((nb, 3)), np.empty((nb, 3)), np.empty(nb, np.int32)) for _ in range(2)]
        for b in bufs:
            for a in b:
                G.host_register(a)
        for s in range(4):  # capture the single-step graphs (both spectrum parities) before the timed steps
            e.run_async(1)
            e.atoms_get_async(bufs[s & 1], s & 1)
        e.wait_slot(1)
        t1 = time.perf_counter()
        for s in range(k):
            e.run_async(1)
            e.atoms_get_async(bufs[s & 1], s & 1)
            if s:
                e.wait_slot((s - 1) & 1)  # step s - 1's beads are in host memory
        e.wait_slot((k - 1) & 1)
        out = e.grid_get("phi")
        t2 = time.perf_counter()
        for _ in range(k):
            e.run(1)
            e.atoms_get()
        t3 = time.perf_counter()
        for b in bufs:
            for a in b:
                G.host_unregister(a)
        steady = world * k / ranks_max(t2 - t1)
        line["e2e"] = {"value": steady, "unit": "steps/s", "h2d_bytes_per_step": 0,
                       "d2h_bytes_per_step": int(nb * (3 * 8 * 3 + 4) + out.size * 4 / k),
                       "setup_s": t1 - t0, "setup_h2d_bytes": int(phi_host.size * 4 + xs.size * 8 + nb * 12),
                       "steps": k, "blocking_read_value": world * k / ranks_max(t3 - t2),
                       "note": "steady state: %d steps, each enqueued (phafd_run_async(ctx, 1)) with a read of its "
                               "beads' x, ux, F and image flags into page-locked host memory "
                               "(phafd_atoms_get_async), the host waiting for step s's read while step s + 1 runs; "
                               "phi read after the last; blocking_read_value: each step phafd_run(ctx, 1) then "
                               "phafd_atoms_get; set-up (context, state uploaded from host arrays, first step with "
                               "list build and graph capture) timed apart as setup_s, and four pipelined steps that "
                               "capture the single-step graphs before the timed ones" % k}
        e.close()

    # FP32 production path against the FP64 path and the FP64 oracle from the
    # same state and the same Philox noise, 50 steps: S(k) error, with the FP32
    # stages taken relative to the mean of phi switched off one by one
    if rank == 0 and world == 1 and not args.no_e2e:
        line["fp32_vs_fp64"] = precision_check(cfg, chains, local, 50)

    if rank == 0 and world == 1 and not args.no_learned and args.workload == WORKLOAD:
        try:
            line["learned"] = learned_vs_plain(args, 256)
        except Exception as ex:  # the step numbers above stand without it
            line["learned"] = {"error": str(ex)[:300]}

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, dt, threads = cpu_baseline_oracle(cfg, chains, 3)
        line["cpu_baseline"] = {"value": v, "unit": "steps/s", "cores": threads, "kind": "port",
                                "cpu_model": cpu_model(), "mpi_ranks": 1,
                                "sample": "3 steps of %s (FP64 oracle restatement; grid loops on %d threads, bead "
                                          "loops on one) after its set-up" % (args.workload, threads)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if torch_dist:
        torch_dist.destroy_process_group()
    return 0


def sk_shells(phi):
    """shell-averaged S(k) of a real cubic field (k = 0 left out)"""
    from tests.helpers import shell_sk
    return shell_sk(phi)


def precision_check(cfg, chains, device, steps):
    import numpy as np
    from phafd_gb300 import workloads as W
    from phafd_gb300.gpu import PhafdGPU

    def sk_err(a, b):
        m = b[1:] > 0
        return float(np.max(np.abs(a[1:][m] - b[1:][m]) / b[1:][m]))

    def run(prec, nsteps, fh=False, fft=True):
        g = PhafdGPU(precision=prec, device=device, schedule="resident")
        W.apply(g, cfg, chains=chains)
        g.set_fp32_centering(fh=fh, fft=fft)
        g.setup()
        g.run(nsteps)
        out = g.structure_factor(cfg["n"] // 2)[0], g.grid_get("phi")
        g.close()
        return out

    out = {"steps": steps}
    s64, p64 = run(64, steps)
    s32, p32 = run(32, steps)
    out["sk_rel_err_max"] = sk_err(s32, s64)
    out["phi_max_abs_err"] = float(np.max(np.abs(p32 - p64)))
    out["mass_err"] = float(abs(p32.mean() - p64.mean()))
    # the FP32 error budget: S(k) error with the stages relative to the mean
    # of phi switched off one at a time, and the representation floor (the
    # FP32 rounding of the initial field, no step)
    budget = {"transforms_centered (default)": out["sk_rel_err_max"]}
    for name, fh, fft in (("fh_and_transforms_centered", True, True), ("fh_centered_only", True, False),
                          ("none_centered", False, False)):
        budget[name] = sk_err(run(32, steps, fh, fft)[0], s64)
    budget["initial_field_rounding"] = sk_err(run(32, 0)[0], run(64, 0)[0])
    out["budget"] = budget
    # the FP32 path against the FP64 oracle itself (the reference's CPU algorithm)
    try:
        from oracle import oracle as OR
        from oracle.oracle import Oracle
        OR.set_threads(OR.host_threads())
        o = Oracle()
        W.apply(o, cfg, chains=chains)
        o.setup()
        o.run(steps)
        po = o.grid_get("phi")
        del o
        out["sk_rel_err_vs_oracle"] = sk_err(sk_shells(p32), sk_shells(po))
        out["fp64_gpu_phi_rel_err_vs_oracle"] = float(np.abs(p64 - po).max() / np.abs(po).max())
    except Exception as ex:
        out["oracle_error"] = str(ex)[:200]
    # bead forces of one pair evaluation at identical positions (FP32 pair
    # arithmetic with compensated sums against FP64)
    try:
        forces = {}
        for prec in (32, 64):
            g = PhafdGPU(precision=prec, device=device, schedule="resident")
            W.apply(g, cfg, chains=chains)
            g.setup()  # lists built and the gradient of phi current
            g.stage_pairs()  # the step's own pair launch, forces assigned
            forces[prec] = g.atoms_get()[2]
            g.close()
        d = forces[32] - forces[64]
        out["force_rel_err"] = float(np.linalg.norm(d) / np.linalg.norm(forces[64]))
        out["force_max_abs_err"] = float(np.abs(d).max())
    except Exception as e:  # the step numbers above stand without it
        out["force_rel_err"] = None
        out["force_error"] = str(e)[:200]
    return out


def run_ensemble(args):
    """Ragged 48-replica ensemble (grids 96^3/128^3/160^3, 2k-20k beads):
    every replica enqueued, all overlapping on one GPU; value is replica
    steps per second."""
    # 48 contexts x 3 streams: more hardware work queues than the default 8
    # keep their graphs from queueing behind one another (read when the CUDA
    # runtime starts, which has not happened yet in this process)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    from phafd_gb300 import build as B
    B.build()
    from phafd_gb300.ensemble import Ensemble, ensemble_configs
    cfgs = ensemble_configs(48)
    ens = Ensemble(cfgs, precision=32)
    ens.run(max(args.warmup, 3))
    import ctypes
    t0 = time.perf_counter()
    ens.run(args.steps)
    dt = time.perf_counter() - t0
    rs = ens.replica_steps(args.steps)
    sizes = {}
    for c in cfgs:
        sizes[c["n"]] = sizes.get(c["n"], 0) + 1
    line = {"metric": "replica steps/s, ragged 48-replica ensemble", "value": rs / dt, "unit": "replica-steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": 1000 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "ensemble48", "replicas": len(cfgs), "grids": sizes,
                       "beads_total": int(sum(c["nchains"] * c["chain_len"] for c in cfgs)),
                       "timing": "host wall clock around enqueue of all replicas + synchronize"}}
    print(json.dumps(line), flush=True)
    ens.close()
    return 0


def learned_vs_plain(args, n_eval):
    """Learned propagator: train the spectral neural operator on trajectories
    of the plain FP32 integrator at 128^3 (4k-16k beads, chi in [2.5, 3.5],
    phi0 in [0.35, 0.5]), then on a held-out seed at n_eval^3 time the plain
    path and the surrogate path (macro step of K = 20 substeps, judged every
    100 substeps) over the same substeps and report their S(k) errors against
    the plain path.  Returns the measurements as a dict."""
    import numpy as np
    import torch
    from phafd_gb300 import surrogate as S
    rng = np.random.default_rng(2024)
    specs = [(128, int(rng.integers(4000, 16001)), rng.uniform(2.5, 3.5), rng.uniform(0.35, 0.5), 5000 + i)
             for i in range(args.traj)]
    t0 = time.perf_counter()
    data = S.generate(specs, samples=2, burn=200, gap=100)
    t_gen = time.perf_counter() - t0
    net = S.new_network((128, 128, 128), train=True, seed=1)
    net.set_norm(S.norm_from(*data))
    t0 = time.perf_counter()
    hist = S.train(net, data, epochs=args.epochs, lr=1e-3, batch=8)
    t_train = time.perf_counter() - t0
    params, norm = net.get_params(), net.norm.copy()
    gain_train = S.gain(net, data)
    net.close()
    del data
    held_specs = [(128, 10000, 3.0, 0.42, 9001), (128, 6000, 2.8, 0.38, 9002)]
    held = S.generate(held_specs, samples=2, burn=200, gap=100, workers=2)
    inf128 = S.new_network((128, 128, 128), params=params, norm=norm)
    gain_held = S.gain(inf128, held)
    inf128.close()
    del held
    # held-out evaluation run
    nb = 10000 if n_eval == 128 else 32000
    cfg = S.traj_cfg(n_eval, nb, 3.0, 0.4, 9100)
    chains = S.make_chains([cfg], 1)[0]
    net = S.new_network((n_eval,) * 3, params=params, norm=norm)
    horizon = 200
    herr = S.horizon_error(cfg, chains, net, horizon)
    nsub = max(args.steps, 200) // 100 * 100
    plain = S.sim(cfg, chains, noise=True)
    plain.run(max(args.warmup, 3))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain.run(nsub)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    plain.close()
    run = S.Runner(cfg, chains, net, judge_every=100, sk_bound=SK_BOUND, mass_bound=MASS_BOUND)
    run.run(100)  # warm-up window (judge + 5 macro steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run.run(nsub)
    torch.cuda.synchronize()
    t_sur = time.perf_counter() - t0
    judged = [{"step": j[0], "sk_err": j[1], "mass_err": j[2], "accepted": bool(j[3])} for j in run.judged]
    phase_s = dict(run.times)
    run.close()
    # the same judged run with the linearised macro step alone
    lin = S.Runner(cfg, chains, None, judge_every=100, sk_bound=SK_BOUND, mass_bound=MASS_BOUND)
    lin.run(100)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lin.run(nsub)
    torch.cuda.synchronize()
    t_lin = time.perf_counter() - t0
    judged_lin = [{"step": j[0], "sk_err": j[1], "accepted": bool(j[3])} for j in lin.judged]
    lin.close()
    # network inference alone, CUDA events around the call
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rho = torch.zeros((n_eval,) * 3, device="cuda")
    corr = torch.empty_like(rho)
    phi = torch.full_like(rho, 0.4)
    net.infer(phi.data_ptr(), rho.data_ptr(), 3.0, corr.data_ptr())
    torch.cuda.synchronize()
    ev0.record()
    for _ in range(5):
        net.infer(phi.data_ptr(), rho.data_ptr(), 3.0, corr.data_ptr())
    ev1.record()
    torch.cuda.synchronize()
    infer_ms = ev0.elapsed_time(ev1) / 5
    net.close()
    v_sur, v_plain = nsub / t_sur, nsub / t_plain
    return {
        "learned_steps_per_s": v_sur, "steps": nsub, "ms_per_step": 1000 * t_sur / nsub,
        "config": {"grid": [n_eval] * 3, "beads": W_nbeads(cfg), "K": S.K_SUB,
                   "judge_every": 100, "judge_sk_bound": SK_BOUND, "judge_mass_bound": MASS_BOUND,
                   "train_grid": [128] * 3, "train_trajectories": args.traj,
                   "train_samples": 2 * args.traj, "epochs": args.epochs,
                   "timing": "host wall clock around run(), synchronised; includes the judge windows"},
        "plain_steps_per_s": v_plain, "speedup_vs_plain": v_sur / v_plain,
        "linear_macro_steps_per_s": nsub / t_lin, "linear_macro_speedup_vs_plain": (nsub / t_lin) / v_plain,
        "judge_linear_macro": judged_lin,
        "horizon_substeps": horizon, "errors_vs_plain": herr,
        "macro_error_rel": {"train": gain_train, "held_out_128": gain_held, "linear_step_alone": 1.0},
        "judge": judged, "train_loss": hist, "seconds": {"generate": t_gen, "train": t_train},
        "timed_phase_seconds": phase_s, "network_infer_ms": infer_ms,
    }


def run_learned(args):
    """The learned-vs-plain measurement as a line of its own (learned128 /
    learned256)."""
    from phafd_gb300 import build as B
    B.build()
    n_eval = 256 if args.workload == "learned256" else 128
    r = learned_vs_plain(args, n_eval)
    cfg = dict(r.pop("config"), workload=args.workload)
    line = {"metric": "steps/s, learned macro step vs plain FP32 step", "value": r["learned_steps_per_s"],
            "unit": "steps/s", "n_gpus": 1, "steps": r["steps"], "warmup": max(args.warmup, 3),
            "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 network, f32 field", "data": "synthetic", "config": cfg}
    line.update(r)
    print(json.dumps(line), flush=True)
    return 0


# judge bounds of the learned macro step against K plain substeps from the
# same state: relative S(k) error (max over shells) and mass error
SK_BOUND = 5e-3
MASS_BOUND = 1e-6


def W_nbeads(cfg):
    return cfg["nchains"] * cfg["chain_len"]


def fno_bytes_per_inference(n):
    """Compulsory HBM bytes of one network inference on an n^3 grid: lift
    (phi, rho in; v0 and its x-stage partials out), four layers (v in, x-inverse
    rows in, v out, x-stage partials out for the next layer), the y stages of
    the spectral branches, the projection and the centring."""
    N = n ** 3
    halves = max(1, n // 128)
    xst = 16 * 32 * 4 * halves / n          # x-stage partials per node
    rows = 32 * 16 * 2 / n                  # x-inverse input per node
    lift = 8 + xst                          # phi, rho in; x stage of v0 out (v0 is rebuilt in layer 0)
    layer0 = 8 + rows + 64 + xst
    layers12 = 2 * (64 + rows + 64 + xst)
    layer3 = 64 + rows + 4                  # projection folded in: out only
    spectral = 4 * (xst + rows)
    centre = 8
    return N * (lift + layer0 + layers12 + layer3 + spectral + centre)


def run_fno_infer(args):
    """Inference of the spectral neural operator alone (random parameters)."""
    import numpy as np
    import torch
    from phafd_gb300 import build as B
    B.build()
    from phafd_gb300.fno import FNO, init_params
    n = 256 if args.workload == "fno_infer256" else 128
    net = FNO((n, n, n))
    net.set_params(init_params(0, out_scale=1.0))
    net.set_norm(np.array([0.4, 0.02, 0.0, 1.0, 3.0, 0.3, 1e-3, 0.0], np.float32))
    g = torch.Generator(device="cuda").manual_seed(0)
    phi = 0.4 + 0.02 * torch.randn((n, n, n), device="cuda", generator=g)
    rho = torch.relu(torch.randn((n, n, n), device="cuda", generator=g)) * 0.1
    corr = torch.empty_like(phi)
    st = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 3)):
        net.infer(phi.data_ptr(), rho.data_ptr(), 3.0, corr.data_ptr(), stream=st.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        net.infer(phi.data_ptr(), rho.data_ptr(), 3.0, corr.data_ptr(), stream=st.cuda_stream)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    peak, kind = measured_peak()
    nbytes = fno_bytes_per_inference(n)
    line = {"metric": "network inferences/s (spectral neural operator, %d^3)" % n, "value": 1000.0 / ms,
            "unit": "inferences/s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 activations, f32 accumulate", "data": "synthetic",
            "config": {"workload": args.workload, "grid": [n] * 3, "channels": 32, "layers": 4, "modes": 16},
            "roofline": {"bound": "hbm", "achieved": nbytes / (ms / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": nbytes / (ms / 1000.0) / 1e9 / peak, "peak_kind": kind, "bytes": nbytes}}
    print(json.dumps(line), flush=True)
    net.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ensemble48":
        return run_ensemble(args)
    if args.workload in ("learned128", "learned256"):
        return run_learned(args)
    if args.workload in ("fno_infer128", "fno_infer256"):
        return run_fno_infer(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())

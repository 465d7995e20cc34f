"""Benchmark of the GB300 affine-body contact step.

Workload: the 1024-body icosphere pile (16 x 16 x 4 grid of subdivision-3 icospheres,
radius 0.5, spacing 1.1, seeded rotation / jitter / velocity; dt 0.01, dhat 1e-3,
mu 0.1, Newton tol 1e-4), started from its committed contact-rich checkpoint
(adb_gb300/data/pile_ckpt.npz, written by adb_gb300/data/make_checkpoint.py) so that
every timed frame carries the full contact load. A step is one frame
(ABD::implicit_euler). Metric: frames/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

gb300 arm: W untimed frames, then K frames timed with CUDA events on the engine's
stream (value, state resident in HBM), then the same K frames again through the public
C ABI with host buffers (e2e: pinned host state -> device, step, device -> host every
frame), then one profiled pass (up to 5 frames) for the per-kernel roofline. The CPU
baseline times the oracle on the first Newton iterations of the first timed frame. N > 1 runs N independent
replicas (one per GPU; the pile does not shard): value = total frames/s of all ranks
over the max-over-ranks time. The line also carries the pile's 200-frame run from rest
(pile_200), the 200-link chain, the batched and the differentiable-rollout workloads.
reference arm: the CPU restatement of the reference (oracle/, OpenMP on all host
cores) on the same checkpoint, each step one frame, bounded by a time budget.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s, 1024-body pile GPU vs CPU ref; batched vs looped scenes/s at tol"
CKPT = os.path.join(ROOT, "adb_gb300", "data", "pile_ckpt.npz")
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "traffic.md")


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def dist_barrier(world):
    """Host barrier of the ranks (abd_step returns after synchronising its stream, so a
    host barrier orders the ranks' device work too)."""
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(x, world):
    """Largest x over the ranks (the job's time is its slowest rank's)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def pile_workload():
    from adb_gb300 import scene as S
    sc = S.sphere_pile(seed=0)
    cfg = S.workload_config("pile")
    q0, qd, frame = sc.q0, sc.dqdt, 0
    if os.path.exists(CKPT):
        z = np.load(CKPT)
        q0, qd, frame = z["q0"], z["qdot"], int(z["frame"])
    return sc, cfg, q0, qd, frame


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap,memory.used")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        mem = [float(s[7]) for s in self.samples if len(s) > 7 and s[7].replace(".", "").isdigit()]
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples),
                "mem_used_gib": round(max(mem) / 1024.0, 2) if mem else None}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def ncu_per_unit(kernel, key="traffic_per_unit"):
    """A per-work-unit figure of `kernel` from the committed ncu summary, if any: DRAM
    bytes (`traffic_per_unit`) or executed FP64 flops (`fp64_flops_per_unit`)."""
    if not os.path.exists(PROFILE_TRAFFIC):
        return None
    for line in open(PROFILE_TRAFFIC):
        if line.startswith(key) and line.split("=")[0].split()[-1] == kernel:
            try:
                return float(line.split("=")[1].split()[0])
            except Exception:
                return None
    return None


def batched_vs_looped(frames=5, warm_frames=30, n_scenes=256, loop_budget_s=30.0, rank=0, world=1):
    """The batched half of the metric: 256 independent scenes stepped in one handle
    against the same scenes stepped one handle at a time, from the same state, at the same
    Newton tolerance. Both sides are timed on the wall clock around the step calls (every
    step call ends with a stream synchronisation). The looped side steps the scenes in
    order until its time budget is spent (at least 8 scenes); its rate is the scene-frames
    it finished over its time, and its final states are compared bit for bit with the
    batched run. With several ranks the batch is sharded by scene (scene k on rank k %
    world, no exchange): each rank steps its shard in one handle, the batched rate is all
    scenes over the slowest rank's time, and each rank loops its own shard's scenes."""
    from adb_gb300 import scene as S
    from adb_gb300.abd import ABD
    full = S.batched_scenes(n_scenes=n_scenes, seed=0)
    sc = full.scenes_of_rank(rank, world) if world > 1 else full
    cfg = S.workload_config("batched")
    bat = ABD(sc, cfg)
    bat.step(warm_frames)                     # falling bodies reach their first contacts
    q0, qd = bat.state()
    it0 = bat.scene_stats()["iter"].copy()
    dist_barrier(world)
    t0 = time.perf_counter()
    bst = bat.step(frames)
    t_bat = dist_max(time.perf_counter() - t0, world)
    bq, bqd = bat.state()
    bat.close()
    ranges = sc.scene_ranges()
    t_loop, looped, same = 0.0, 0, True
    for k, (b0, b1) in enumerate(ranges):
        if looped >= 8 and t_loop > loop_budget_s:
            break
        h = ABD(sc.body_range(b0, b1), cfg)
        h.set_state(q0[b0:b1], qd[b0:b1])
        h.iter = int(it0[k])
        t0 = time.perf_counter()
        h.step(frames)
        t_loop += time.perf_counter() - t0
        q, qdd = h.state()
        same = same and bool(np.array_equal(q, bq[b0:b1]) and np.array_equal(qdd, bqd[b0:b1]))
        h.close()
        looped += 1
    bat_rate = len(full.scene_ranges()) * frames / t_bat
    loop_rate = dist_sum(looped * frames / t_loop, world)   # the ranks loop at the same time
    same = dist_sum(0.0 if same else 1.0, world) == 0.0
    return {"scenes": len(full.scene_ranges()), "bodies": full.n_bodies, "vertices": full.n_vertices,
            "frames": frames, "ranks": world,
            "start": "frame %d of the seeded batch" % warm_frames,
            "batched_scenes_per_s": bat_rate, "looped_scenes_per_s": loop_rate,
            "looped_sample": "first %d of %d scenes (%.1f s)" % (looped, len(ranges), t_loop),
            "speedup": bat_rate / loop_rate, "bitwise_equal_to_looped": same,
            "newton_iters": bst.newton_iters, "max_pt": bst.n_pt, "max_ee": bst.n_ee}


def adjoint_cost(n_steps=100, every=10):
    """Forward and backward time of the differentiable-rollout workload: 64 subdivision-2
    icospheres (4 x 4 x 4 grid, spacing 1.2), mu 0.3 as a learnable scalar, n_steps frames
    at dt 0.01 with a state checkpoint every `every` frames; loss = sum of squared distances
    of the final body centres to seeded targets; gradients with respect to the 64 x 12
    initial affine velocities and mu. The backward pass recomputes the frames between
    checkpoints and solves one adjoint system per frame. Timed on the wall clock."""
    import torch
    from adb_gb300 import scene as S
    from adb_gb300.abd import ABD
    from adb_gb300.adjoint import rollout
    sc = S.diff_grid(seed=0)
    cfg = S.workload_config("diff")
    tgt = torch.tensor(S.diff_targets(sc.n_bodies, seed=0))
    sim = ABD(sc, cfg)
    v0 = torch.zeros(sc.q0.shape, dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(cfg.mu, dtype=torch.float64, requires_grad=True)
    t0 = time.perf_counter()
    qT, _ = rollout(sim, torch.tensor(sc.q0), v0, mu, n_steps, every)
    t_fwd = time.perf_counter() - t0
    loss = ((qT[:, :3] - tgt) ** 2).sum()
    t0 = time.perf_counter()
    loss.backward()
    t_bwd = time.perf_counter() - t0
    sim.close()
    return {"scene": "64 icosphere-s2 grid, mu %.1f, seeded targets" % cfg.mu, "frames": n_steps,
            "checkpoint_every": every, "forward_s": t_fwd, "backward_s": t_bwd,
            "backward_over_forward": t_bwd / t_fwd, "dL_dmu": float(mu.grad)}


def kernel_roofline(sim, frames, fp64_peak):
    """Profiled pass of `frames` frames from the simulation's current state: per-kernel
    device time (CUDA events around every launch on the engine's stream), and for the
    dominant kernel its algorithmic bytes per launch over its average launch time against
    the measured HBM copy bandwidth, its DRAM traffic per launch (ncu bytes per unit from
    the committed profile summary times the units per launch) and its FP64 rate."""
    sim.profile(True)
    pst = sim.step(frames)
    kt = sim.kernel_times()
    sim.profile(False)
    tot = sum(v["ms"] for v in kt.values())
    dom = max(kt, key=lambda k: kt[k]["ms"])
    d = kt[dom]
    peak, peak_kind = measured_peaks()
    avg_ms = d["ms"] / max(d["launches"], 1)
    bytes_per_launch = d["bytes"] / max(d["launches"], 1)
    achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9 if avg_ms > 0 else 0.0
    tpu = ncu_per_unit(dom)
    traffic = tpu * d["units"] / max(d["launches"], 1) if tpu else None
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": traffic, "avg_launch_ms": avg_ms, "launches": d["launches"],
            "share": d["ms"] / tot if tot else None,
            # kernel time against the device time of the same profiled frames: the rest
            # is the GPU waiting on the host (synchronisations and launches)
            "profiled_frames": frames, "profiled_kernel_ms": tot, "profiled_device_ms": pst.device_ms}
    # the dominant kernels of this FP64 path are bound by FP64 issue, not by HBM: their
    # FP64 rate (flops per unit from one ncu capture x units per launch / live launch
    # time) against the measured FP64 FMA peak
    fpu = ncu_per_unit(dom, "fp64_flops_per_unit")
    fp64_roof = None
    if fpu and avg_ms > 0:
        gf = fpu * d["units"] / max(d["launches"], 1) / (avg_ms * 1e-3) / 1e9
        fp64_roof = {"achieved_gflops": gf, "peak_gflops": fp64_peak, "frac": gf / fp64_peak,
                     "flops_per_unit": fpu, "source": "executed DFMA x2 + DADD + DMUL per unit (ncu), live time"}
    return roof, fp64_roof, kt


def chain_line(frames=300, fp64_peak=None):
    """The 200-link chain (48 x 24 tori, dt 0.005, dhat 1e-4, mu 0.2, ground off, link 0
    static) over its first `frames` frames from rest: timed with the state resident (CUDA
    events), again through the C ABI with host buffers every frame (e2e), then a profiled
    pass of 5 frames from the state at 80% of the run for the dominant kernel. The CPU
    restatement is timed on one frame at each of three states of the GPU trajectory (20%,
    50% and 80% of the run; the early frames carry no contact and are cheaper) on all host
    cores, and its rate is the inverse of their mean frame time."""
    import ctypes as C
    from adb_gb300 import _lib as L
    from adb_gb300 import scene as S
    from adb_gb300.abd import ABD
    from oracle import oracle as O
    sc, cfg = S.torus_chain(seed=0), S.workload_config("chain")
    sim = ABD(sc, cfg)
    q0, qd = sim.state()
    marks = {int(frames * 0.2), int(frames * 0.5), int(frames * 0.8)}
    states = {}
    dev_ms, newton, trials, mpt, mee, capped = 0.0, 0, 0, 0, 0, []
    for f in range(frames):
        if f in marks:
            states[f] = sim.state() + (sim.iter,)
        st = sim.step(1)
        if cfg.max_iter_frame and st.newton_iters >= cfg.max_iter_frame:
            capped.append(f + 1)
        dev_ms += st.device_ms
        newton += st.newton_iters
        trials += st.ls_trials
        mpt, mee = max(mpt, st.n_pt), max(mee, st.n_ee)
    value = frames / (dev_ms / 1000.0)
    sim.set_state(q0, qd)
    sim.iter = 0
    lib = L.lib()
    hq, hqd = np.ascontiguousarray(q0), np.ascontiguousarray(qd)
    outq, outqd = np.zeros_like(hq), np.zeros_like(hqd)
    est = L.AbdFrameStats()
    t0 = time.perf_counter()
    for _ in range(frames):
        lib.abd_set_state(sim._h, L.dptr(hq), L.dptr(hqd))
        lib.abd_step(sim._h, 0.0, 1, C.byref(est))
        lib.abd_get_state(sim._h, L.dptr(outq), L.dptr(outqd))
        hq, hqd = outq.copy(), outqd.copy()
    e2e = frames / (time.perf_counter() - t0)
    late = max(marks)
    sim.set_state(states[late][0], states[late][1])
    sim.iter = states[late][2]
    roof, fp64_roof, kt = kernel_roofline(sim, 5, fp64_peak or 0.0)
    sim.close()
    cores = os.cpu_count() or 1
    secs = []
    for f in sorted(marks):
        orc = O.OracleSim(sc, cfg, n_threads=cores)
        orc.set_state(states[f][0], states[f][1])
        orc.iter = states[f][2]
        t0 = time.perf_counter()
        orc.step(1)
        secs.append(time.perf_counter() - t0)
    return {"workload": "chain-200 torus 48x24, frames 1-%d from rest" % frames, "bodies": sc.n_bodies,
            "vertices": sc.n_vertices, "dt": cfg.dt, "dhat": cfg.dhat, "mu": cfg.mu, "value": value,
            "unit": "frames/s", "steps": frames, "ms_per_step": dev_ms / frames,
            "e2e": {"value": e2e, "unit": "frames/s", "h2d_bytes_per_step": hq.nbytes + hqd.nbytes,
                    "d2h_bytes_per_step": outq.nbytes + outqd.nbytes},
            "roofline": roof, "fp64": fp64_roof,
            "frame_stats": {"newton_iters": newton, "ls_trials": trials, "max_pt": mpt, "max_ee": mee,
                            "frames_at_newton_cap": capped, "newton_cap_per_frame": cfg.max_iter_frame},
            "kernel_ms_profiled_5_frames": {k: round(v["ms"], 3) for k, v in
                                            sorted(kt.items(), key=lambda kv: -kv[1]["ms"]) if v["ms"] > 0},
            "cpu_baseline": {"value": len(secs) / sum(secs), "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": "frames %s of the GPU trajectory, one each, all host cores (%s s)" % (
                                 ", ".join(str(f + 1) for f in sorted(marks)),
                                 ", ".join("%.2f" % x for x in secs))}}


def pile_run_line(frames=200):
    """The pile's own 200-frame run: the seeded 1024-icosphere pile from rest (bodies
    falling, first contacts, compression), frames 1-`frames`, each frame timed with CUDA
    events on the engine's stream with the state resident. Frames whose lagged friction
    makes the Newton iteration cycle stop at the workload's per-frame cap and are listed."""
    from adb_gb300 import scene as S
    from adb_gb300.abd import ABD
    sc, cfg = S.sphere_pile(seed=0), S.workload_config("pile")
    sim = ABD(sc, cfg)
    dev_ms, newton, trials, capped, mpt, mee = 0.0, 0, 0, [], 0, 0
    t0 = time.perf_counter()
    for f in range(frames):
        st = sim.step(1)
        if cfg.max_iter_frame and st.newton_iters >= cfg.max_iter_frame:
            capped.append(f + 1)
        dev_ms += st.device_ms
        newton += st.newton_iters
        trials += st.ls_trials
        mpt, mee = max(mpt, st.n_pt), max(mee, st.n_ee)
    wall = time.perf_counter() - t0
    sim.close()
    return {"workload": "pile-1024 icosphere-s3, frames 1-%d from rest" % frames, "value": frames / (dev_ms / 1000.0),
            "unit": "frames/s", "steps": frames, "ms_per_step": dev_ms / frames, "wall_s": wall,
            "frame_stats": {"newton_iters": newton, "ls_trials": trials, "max_pt": mpt, "max_ee": mee,
                            "frames_at_newton_cap": capped, "newton_cap_per_frame": cfg.max_iter_frame}}


def cpu_baseline_sample(sc, cfg, q0, qd, newton_per_frame, ls_per_frame, sample_iters=6):
    """The CPU restatement on all host cores, timed on a bounded sample of one frame.

    The sample is the first `sample_iters` Newton iterations of the frame that starts from
    (q0, qd). Its time splits into the Newton part (assembly, solve, step bound) per
    iteration and the line search per trial; frames/s is scaled from those by the Newton
    iterations and line-search trials per frame the GPU run took on the same frames (the
    two paths take identical counts, which the parity tests check)."""
    import dataclasses
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    c2 = dataclasses.replace(cfg, max_iter=sample_iters)
    sim = O.OracleSim(sc, c2, n_threads=cores)
    sim.set_state(q0, qd)
    sim.iter = 0
    t0 = time.perf_counter()
    st = sim.step(1)
    secs = time.perf_counter() - t0
    its, trials = max(st.newton_iters, 1), max(st.ls_trials, 1)
    t_newton = (st.t_ipc + st.t_solver + st.t_ccd) / its
    t_trial = st.t_ls / trials
    frame_s = newton_per_frame * t_newton + ls_per_frame * t_trial
    return 1.0 / frame_s, cores, its, trials, secs


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sc, cfg, q0, qd, frame = pile_workload()
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    sim = O.OracleSim(sc, cfg, n_threads=cores)
    sim.set_state(q0, qd)
    budget = float(os.environ.get("ABD_REF_BUDGET_S", "100"))
    t0 = time.perf_counter()
    n = 0
    # each step is one frame; the run stops at the time budget (at least one frame)
    for _ in range(max(1, args.steps)):
        st = sim.step(1)
        n += 1
        if st.status != 0 or time.perf_counter() - t0 > budget:
            break
    dt = time.perf_counter() - t0
    v = n / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": n, "warmup": 0, "ms_per_step": 1000.0 * dt / n, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "pile-1024 icosphere-s3 from frame-%d checkpoint" % frame, "bodies": sc.n_bodies,
                       "vertices": sc.n_vertices, "dt": cfg.dt, "dhat": cfg.dhat, "mu": cfg.mu, "tol": cfg.tol},
            "cpu_baseline": {"value": v, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": "%d frame(s) of the pile from the checkpoint, all host cores" % n},
            "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args):
    rank, world, local = dist_env()
    import ctypes as C

    if world > 1:
        # one replica per GPU: this rank's library sees only its own device
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        os.environ["CUDA_VISIBLE_DEVICES"] = vis.split(",")[local] if vis else str(local)
        import torch.distributed as dist
        dist.init_process_group("gloo")
    import __graft_entry__ as G
    G.build()
    from adb_gb300 import _lib as L
    from adb_gb300.abd import ABD, measure_fp64_gflops

    sc, cfg, q0, qd, frame = pile_workload()
    sim = ABD(sc, cfg)

    def barrier():
        dist_barrier(world)

    def max_over_ranks(x):
        return dist_max(x, world)

    # ---- value: W untimed frames, then K frames with the state resident on the device ----
    # warm-up frames from the checkpoint, then back to it: the timed frames are the
    # checkpoint's next frames, the same window the reference arm times
    sim.set_state(q0, qd)
    it0 = sim.iter
    if args.warmup:
        sim.step(args.warmup)
    sim.set_state(q0, qd)
    sim.iter = it0
    start_q, start_qd = q0, qd
    barrier()
    with ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]) if world > 1 else 0) as clk:
        st = sim.step(args.steps)
    barrier()
    dev_s = max_over_ranks(st.device_ms / 1000.0)
    value = world * args.steps / dev_s
    clocks = clk.summary()

    # ---- e2e: same frames through the public API with host buffers ----
    lib = L.lib()
    sim.iter = it0
    hq = np.ascontiguousarray(start_q)
    hqd = np.ascontiguousarray(start_qd)
    outq = np.zeros_like(hq)
    outqd = np.zeros_like(hqd)
    h2d = hq.nbytes + hqd.nbytes
    d2h = outq.nbytes + outqd.nbytes
    barrier()
    t0 = time.perf_counter()
    est = L.AbdFrameStats()
    for k in range(args.steps):
        lib.abd_set_state(sim._h, L.dptr(hq), L.dptr(hqd))
        lib.abd_step(sim._h, 0.0, 1, C.byref(est))
        lib.abd_get_state(sim._h, L.dptr(outq), L.dptr(outqd))
        hq, hqd = outq.copy(), outqd.copy()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    barrier()
    e2e = world * args.steps / e2e_s

    # ---- per-kernel device time (separate profiled pass over the same frames) ----
    sim.set_state(start_q, start_qd)
    sim.iter = it0
    fp64_peak = measure_fp64_gflops()
    roof, fp64_roof, kt = kernel_roofline(sim, min(args.steps, 5), fp64_peak)

    # the batched half runs on every rank (sharded by scene); rank 0 reports it
    batched = None if args.no_batched else batched_vs_looped(rank=rank, world=world)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded icosphere pile, no dataset)",
            "config": {"workload": "pile-1024 icosphere-s3 from frame-%d checkpoint" % frame,
                       "bodies": sc.n_bodies, "vertices": sc.n_vertices, "dt": cfg.dt, "dhat": cfg.dhat,
                       "mu": cfg.mu, "tol": cfg.tol, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "per-frame working set (positions, primitive boxes, pair records) >> 129 MB L2"},
            "clocks": clocks,
            "e2e": {"value": e2e, "unit": "frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(st.kernel_launches),
            "roofline": roof,
            "fp64": {"peak_gflops_measured": fp64_peak, "dominant_kernel": fp64_roof},
            "frame_stats": {"newton_iters": st.newton_iters, "ls_trials": st.ls_trials, "pcg_iters": st.pcg_iters,
                            "max_pt": st.n_pt, "max_ee": st.n_ee, "max_vg": st.n_vg,
                            "algorithmic_GB": st.bytes_moved / 1e9},
            "kernel_ms": {k: round(v["ms"], 3) for k, v in sorted(kt.items(), key=lambda kv: -kv[1]["ms"])
                          if v["ms"] > 0},
            "autotune": sim.autotune_info(),
        }
        if not args.no_batched:
            line["pile_200"] = pile_run_line()
            line["chain"] = chain_line(fp64_peak=fp64_peak)
            line["batched"] = batched
            try:
                line["adjoint"] = adjoint_cost()
            except ImportError as ex:  # torch missing on this host
                line["adjoint"] = {"unavailable": str(ex)}
        if world == 1 and not args.no_cpu_baseline:
            npf = st.newton_iters / max(args.steps, 1)
            lpf = st.ls_trials / max(args.steps, 1)
            v, cores, its, trials, secs = cpu_baseline_sample(sc, cfg, start_q, start_qd, npf, lpf)
            line["cpu_baseline"] = {"value": v, "unit": "frames/s", "cores": cores, "kind": "port",
                                    "sample": ("first %d Newton iterations (%d line-search trials) of the first "
                                               "timed frame (%.1f s), scaled per phase to %.2f iterations and %.2f "
                                               "trials per frame" % (its, trials, secs, npf, lpf))}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()

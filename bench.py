"""Benchmark: free-wake timesteps/s of the 2-blade hovering rotor.

Workload (one "step" = one free-wake timestep of the full solver): 2-blade
hover rotor, R = 1 m, root cut 0.2R, chord 0.08 m, collective 8 deg,
Omega = 100 rad/s, 1 x 24 rings per blade, dt = 5 deg azimuth, 260 near-wake
rows and wake truncation after 6 revs (432 steps), AM2 predictor-corrector,
Squire viscous core growth.  The timed steps run after the wake has reached
its full truncated size (step > 432): 2 x (260 x 24 rings + 24 + 172
filaments) = 50,264 stored filaments, 13,344 wake nodes, two wake-node
evaluations per step.

value: device time of K steps (inputs resident), CUDA events on the case stream.
e2e:   the same steps through the public C entry point vlm_case_step, one call
       per step: the step's wing kinematics frame host->device, the kernels,
       the step's CT row device->host, wall clock.
--impl reference: the reference algorithm on the host CPU (the C++ oracle,
       all cores) stepping the same case through the same steady-state steps,
       from the state the FP64 GPU solver reaches there (the oracle cannot
       afford the first 432 steps in a bench run; see run_reference).
"""
from __future__ import annotations

import argparse
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

from volcanor_gb300 import cases as C  # noqa: E402

METRIC = "free-wake timesteps/s at <=1e-4 rel CT err vs FP64 GPU; Biot-Savart pairs/s"
WORKLOAD = ("2-blade hover rotor R=1m c=0.08m theta0=8deg Omega=100rad/s 1x24 rings/blade dt=5deg, "
            "260 near-wake rows, truncation at 6 revs (432 steps), AM2, viscous core growth; "
            "steady-state steps (full 50,264-filament wake)")
FULL_WAKE_STEP = 432
RING_FLOP = 176.0  # flop per ring-target pair (4 filaments x 44)
FIL_FLOP = 44.0
PROFILES = Path(__file__).resolve().parent / "profiles"


def profiled_traffic(name: str):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of
    a kernel, from the committed ncu summary profiles/<name>.txt (its line
    'traffic_bytes_per_launch: N'); None if there is none."""
    f = PROFILES / f"{name}.txt"
    try:
        for line in f.read_text().splitlines():
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1].strip()))
    except OSError:
        return None
    return None


class nvtx_range:
    """NVTX push/pop range (lets an ncu capture select the launches inside)."""

    def __init__(self, name: str):
        self.name = name
        self.ok = False

    def __enter__(self):
        try:
            import torch
            torch.cuda.nvtx.range_push(self.name)
            self.ok = True
        except Exception:
            pass
        return self

    def __exit__(self, *a):
        if self.ok:
            import torch
            torch.cuda.nvtx.range_pop()


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

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
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_handoff(c, case_gpu, chunk: int = 256):
    """An oracle (the C++ FP64 restatement of the reference's path, OpenMP
    over targets on all host cores) of case files c, brought to the flow state
    of GPU case_gpu at its iteration (oracle/handoff.py)."""
    from oracle import handoff
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    sim = O.Sim(c.config, c.geom)
    sim.set_sum_chunk(chunk)
    sim.start()
    handoff.load_case_state(sim, case_gpu)
    return sim


def cpu_steps(sim, gpu_rows, seconds: float):
    """Times whole oracle timesteps from its current state (at least one, up
    to `seconds`), and checks their CT rows against the FP64 GPU rows of the
    same steps from the same state (gpu_rows)."""
    times = []
    while len(times) < len(gpu_rows) and (not times or sum(times) < seconds):
        t0 = time.perf_counter()
        sim.step(1)
        times.append(time.perf_counter() - t0)
    n = len(times)
    ref = sim.ct_hist()[-n:]
    same = bool(np.array_equal(ref, gpu_rows[:n]))
    threads = os.cpu_count() or 1
    return {"value": round(n / sum(times), 4), "unit": "timesteps/s", "cores": threads, "kind": "port",
            "sample": (f"{n} whole timesteps (steps {int(ref[0, 0])}-{int(ref[-1, 0])}) of the same case from the "
                       f"timed window's start state, {sum(times):.1f} s; oracle = C++ FP64 restatement of the "
                       "reference's path with OpenMP over targets (no Fortran compiler for the reference itself)"),
            "ct_rows_bitwise_equal_to_fp64_gpu": same}


def cfg3_rings(M: int, N: int, seed: int = 0):
    """Isolated-kernel workload: N quadrilateral rings (corner 1 ~ U[0,1]^3,
    edges of length U(0.005, 0.05) in random directions, closed), core radius
    0.002, circulation ~ N(0,1); M targets ~ U[0,1]^3."""
    rng = np.random.default_rng(seed)
    c0 = rng.uniform(0, 1, size=(N, 3))

    def edge():
        v = rng.normal(size=(N, 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        return v * rng.uniform(0.005, 0.05, size=(N, 1))
    e1, e2 = edge(), edge()
    corners = np.stack([c0, c0 + e1, c0 + e1 + e2, c0 + e2], axis=1)
    return corners, np.full((N, 4), 0.002), rng.normal(size=N), rng.uniform(0, 1, size=(M, 3))


def run_kernel_cfg3(prec: int, reps: int, M: int = 1 << 20, N: int = 1 << 18):
    """Ring-target pairs/s of vlm_biot_savart_rings_device on the isolated-kernel
    workload (inputs resident in HBM), CUDA events on torch's current stream."""
    import torch
    from volcanor_gb300 import lib
    corners, rvc, gam, P = cfg3_rings(M, N)
    dev = torch.device("cuda")
    tc = torch.from_numpy(corners).to(dev)
    tr = torch.from_numpy(rvc).to(dev)
    tg = torch.from_numpy(gam).to(dev)
    tp = torch.from_numpy(P).to(dev)
    tv = torch.zeros_like(tp)
    stream = torch.cuda.current_stream().cuda_stream
    call = lambda: lib.biot_savart_rings_device(tc.data_ptr(), tr.data_ptr(), tg.data_ptr(), N, tp.data_ptr(), M,
                                                tv.data_ptr(), prec, stream)
    call()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        call()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    pairs = float(M) * N
    return {"M": M, "N": N, "ms_per_launch": round(ms, 3), "pairs_per_s": pairs / (ms / 1e3),
            "tflops": pairs * RING_FLOP / (ms / 1e3) / 1e12}


def max_over_ranks(x: float, dist=None, device: str = "cuda") -> float:
    """The maximum of x over the ranks of the process group (x itself when
    there is none): the contract's max-over-ranks timing."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job throughput of `world` independent replicas that each did
    units_per_rank units, the slowest in `seconds`."""
    return world * units_per_rank / seconds


def run_ours(args):
    from volcanor_gb300 import lib
    rank, world = env_int("RANK", 0), env_int("WORLD_SIZE", 1)
    local = env_int("LOCAL_RANK", 0)
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    prec = {"fp32near": lib.PREC_FP32_NEAR64, "fp32": lib.PREC_FP32, "fp64": lib.PREC_FP64}[args.precision]
    K, W = args.steps, args.warmup
    nt = FULL_WAKE_STEP + W + 2 * K + 2
    c = C.rotor_2blade_hover(nt=max(nt, 1440))
    case = lib.Case(c.config, c.geom, precision=prec, device=local)
    case.start()
    # reach the steady state, then W warm-up steps
    done = 0
    while done < FULL_WAKE_STEP + W:
        n = min(100, FULL_WAKE_STEP + W - done)
        case.step(n, with_ct=False)
        done += n
    # the state at the start of the timed window: the FP64 GPU form, the
    # accuracy check and the CPU baseline all continue from it
    import tempfile
    tmpdir = tempfile.TemporaryDirectory()
    ck = Path(tmpdir.name) / "window_start.ckpt"
    case.checkpoint_save(ck)
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk, nvtx_range("timed_steps"):
        l0 = lib.launch_count()
        t0 = time.perf_counter()
        rows = case.step(K)
        launches = lib.launch_count() - l0
        wall = time.perf_counter() - t0
        dev_ms = case.last_step_ms()
    if dist:
        dist.barrier()
    dev_ms = max_over_ranks(dev_ms, dist)
    value = replica_rate(K, world, dev_ms / 1e3)
    # e2e: one public-API call per step with host buffers
    e2e_steps = K
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        case.step(1)
    e2e_wall = max_over_ranks(time.perf_counter() - t0, dist)
    e2e = replica_rate(e2e_steps, world, e2e_wall)
    frame_doubles = None
    try:
        nb, nc, ns = case.geti("nb"), case.geti("nc"), case.geti("ns")
        frame_doubles = nb * nc * ns * 27 + nb * ns * 12 + nb * 9 + 10 + 9 * (nb - 1)
    except Exception:
        pass
    # roofline of the dominant kernel on the live steady-state state
    with nvtx_range("profile_eval"):
        ms_l, rp, fp = case.profile_eval(20)
    exec_flops, exec_fils = (float(x) for x in case.get("profileWork"))
    near_pairs = case.geti("nearPairs") if prec == lib.PREC_FP32_NEAR64 else 0
    node_chunks = case.geti("nodeChunks")
    tune = None
    if prec != lib.PREC_FP64:
        t = case.autotune()
        if t.size:
            r = t[-1]
            tune = {"signature": [int(r[0]), int(r[1])], "candidates_timed": int(r[2]),
                    "wake_nodes": {"shape": int(r[3]), "chunks_largest_group": int(r[4]), "ms": round(r[5], 4),
                                   "wave_model_ms": round(r[6], 4)},
                    "collocation_points": {"shape": int(r[7]), "chunks_largest_group": int(r[8]),
                                           "ms": round(r[9], 4), "wave_model_ms": round(r[10], 4)},
                    "note": "FP32 pair kernel alone, live steady-state evaluation; shape 0 = 512 targets/block, "
                            "4 stages, 2 blocks/SM; 1 = 256 targets/block, 3 stages, 3 blocks/SM"}
    flops = RING_FLOP * rp + FIL_FLOP * fp
    achieved = flops / (ms_l / 1e3) / 1e12
    pk = peaks()
    sm_max = pk.get("sm_max_mhz", 2070.0)
    sm_count = lib.device_info(local)[0]
    fp32_peak = sm_count * 128 * 2 * sm_max * 1e6 / 1e12
    clocks = clk.summary()
    # the FP32 CUDA-core peak measured on this device (the library's
    # FMA-chain kernel), with the SM clock sampled while it runs
    with ClockSampler(local) as pclk:
        fp32_meas, fp32_meas_ms = lib.measure_fp32_peak(local, reps=200)
    out = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "timesteps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": round(dev_ms / K, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"fp32near": "f32 pairs + f64 near-field/accumulation", "fp32": "f32 pairs + f64 accumulation",
                  "fp64": "f64"}[args.precision],
        "data": "synthetic (case files generated by volcanor_gb300/cases.py; no dataset)",
        "config": {"workload": WORKLOAD, "precision": args.precision, "l2": "working set < L2; per-step state "
                   "changes every step (no reuse of cached results)", "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e, 3), "unit": "timesteps/s",
                "h2d_bytes_per_step": 8 * frame_doubles if frame_doubles else None, "d2h_bytes_per_step": 80},
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp32-cuda-core", "achieved": round(achieved, 3), "peak": round(fp32_peak, 2),
                     "unit": "TFLOP/s", "frac": round(achieved / fp32_peak, 4),
                     "traffic": profiled_traffic(f"k_partial32_hover2_steady_{args.precision}"),
                     "traffic_note": "DRAM bytes per launch from the ncu capture summarised in "
                                     f"profiles/k_partial32_hover2_steady_{args.precision}.txt; the working set "
                                     "(sources, targets, partials) stays in L2",
                     "kernel": "k_partial32" if prec != lib.PREC_FP64 else "k_partial64",
                     "ms_per_launch": round(ms_l, 4), "ring_pairs_per_launch": rp, "fil_pairs_per_launch": fp,
                     "near_pairs_per_launch": near_pairs, "chunks": node_chunks, "autotune": tune,
                     "executed_tflops": round(exec_flops / (ms_l / 1e3) / 1e12, 3),
                     "executed_frac": round(exec_flops / (ms_l / 1e3) / 1e12 / fp32_peak, 4),
                     "executed_fil_pairs_per_launch": exec_fils,
                     "work_note": "achieved counts the reference's work (176 flop per ring-target pair, 44 per "
                                  "filament-target pair); the lattice form evaluates a filament shared by two "
                                  "rings once, so the kernel executes fewer flops: executed_* (9 per corner "
                                  "vector, 35 per filament evaluated)",
                     "peak_note": "nominal FP32 CUDA-core peak (SMs x 128 lanes x 2 x max SM clock); "
                                  "MEASURED_PEAKS.json has no FP32 figure",
                     "peak_measured": round(fp32_meas, 2),
                     "frac_measured": round(achieved / fp32_meas, 4),
                     "executed_frac_measured": round(exec_flops / (ms_l / 1e3) / 1e12 / fp32_meas, 4),
                     "peak_measured_note": "vlm_measure_fp32_peak: independent FMA chains on every SM, "
                                           f"{fp32_meas_ms:.3f} ms per launch, CUDA events, 200 launches",
                     "peak_measured_clocks": pclk.summary()},
        "clocks": clocks,
        "ct_last": float(rows[-1, 1]),
    }
    out["pairs_per_s"] = round(rp / (ms_l / 1e3), 1)
    if prec != lib.PREC_FP64:
        inc = case.get("incremental").reshape(-1, 9)
        if inc.shape[0]:
            r = inc[-1]
            out["incremental_predicted_wake"] = {
                "signature": [int(r[0]), int(r[1])], "used": bool(r[2]), "changed_records": int(r[3]),
                "moved_nodes": int(r[4]), "record_capacity": int(r[5]), "node_capacity": int(r[6]),
                "records": int(r[7]), "nodes": int(r[8]),
                "note": "predicted-wake velocities = current-wake ones + the changed records' (new - old) sums; "
                        "full sums at the moved nodes only"}
    if rank == 0 and not args.no_accuracy:
        # the plain FP64 GPU form over the same K steps from the same state:
        # its rate, and this precision's CT error against it on the timed
        # window (K steps stay inside the free wake's pre-chaotic horizon)
        f64 = lib.Case(c.config, c.geom, precision=lib.PREC_FP64, device=local)
        f64.checkpoint_load(ck)
        sim = None
        if not args.no_cpu:
            sim = cpu_handoff(c, f64)
        r64 = f64.step(K)
        ms64 = f64.last_step_ms()
        v64 = K / (ms64 / 1e3)
        out["fp64_gpu"] = {"value": round(v64, 3), "unit": "timesteps/s", "ms_per_step": round(ms64 / K, 3),
                           "value_over_fp64": round(value / v64, 2),
                           "note": "plain FP64 GPU form (FP64 pairs, FP64 inverse) over the same K steps from the "
                                   "same start state"}
        rel = np.abs(rows[:, 1] - r64[:, 1]) / np.abs(r64[:, 1])
        # The free wake is chaotic: any change of arithmetic (a reordered
        # FP64 sum included) grows e-fold every ~9 steps on this rotor, so one
        # comparison from one shared state holds to 1e-4 for ~20 steps only.
        # Over the whole timed window the FP64 form is therefore restarted
        # from this precision's own state every SYNC steps (the same timed
        # steps replayed from the window-start checkpoint, bit-identical to
        # the timed rows) and compared over each segment.
        SYNC = 20
        x = lib.Case(c.config, c.geom, precision=prec, device=local)
        x.checkpoint_load(ck)
        seg_err, replay = [], []
        ckj = Path(tmpdir.name) / "segment.ckpt"
        for j in range(0, K, SYNC):
            n = min(SYNC, K - j)
            x.checkpoint_save(ckj)
            a32 = x.step(n)
            replay.append(a32)
            f64.checkpoint_load(ckj)
            a64 = f64.step(n)
            seg_err.append(float(np.max(np.abs(a32[:, 1] - a64[:, 1]) / np.abs(a64[:, 1]))))
        x.close()
        replay = np.concatenate(replay)
        out["accuracy"] = {"ct_max_rel_err_timed_window": max(seg_err), "timed_window_steps": K,
                           "timed_window": [int(rows[0, 0]), int(rows[-1, 0])],
                           "sync_every_steps": SYNC, "segment_errors": [float(f"{e:.3g}") for e in seg_err],
                           "replay_bitwise_equal_to_timed_rows": bool(np.array_equal(replay, rows)),
                           "ct_max_rel_err_unsynced": float(rel.max()),
                           "against": "the FP64 GPU form from the same state, restarted from this precision's state "
                                      "every sync_every_steps steps; unsynced: one FP64 run over the whole window "
                                      "(chaotic divergence past ~20 steps)"}
        if sim is not None:
            out["cpu_baseline"] = cpu_steps(sim, r64, args.cpu_seconds)
        f64.close()
    if rank == 0 and not args.no_accuracy and prec != lib.PREC_FP64:
        # this precision's CT error against the FP64 GPU form over the first
        # revolution (the free wake's pre-chaotic horizon; see the accuracy module)
        ref = lib.Case(c.config, c.geom, precision=lib.PREC_FP64, device=local)
        ref.start()
        a = ref.step(72)[:, 1]
        ref.close()
        x = lib.Case(c.config, c.geom, precision=prec, device=local)
        x.start()
        b = x.step(72)[:, 1]
        x.close()
        out.setdefault("accuracy", {})
        out["accuracy"].update({"ct_max_rel_err_vs_fp64_first_rev": float(np.max(np.abs(b - a) / np.abs(a))),
                                "first_rev_steps": 72,
                                "note": "the full 1440-step comparison is volcanor_gb300/accuracy.py"})
    if not args.no_kernel:
        # the isolated N-body kernel in both FP32 forms (the FP64 form runs
        # ~60x slower on this part: see the bench's fp64 precision)
        for key, kp in (("kernel_rings", lib.PREC_FP32), ("kernel_rings_near64", lib.PREC_FP32_NEAR64)):
            k3 = run_kernel_cfg3(kp, reps=args.kernel_reps)
            k3["frac_of_fp32_peak"] = round(k3["tflops"] / fp32_peak, 4)
            k3["precision"] = "fp32" if kp == lib.PREC_FP32 else "fp32near"
            k3["workload"] = ("isolated kernel: 2^20 targets x 2^18 rings (U[0,1]^3, edges U(0.005,0.05), "
                              "core 0.002)")
            out[key] = k3
    tmpdir.cleanup()
    if rank == 0 and not args.no_batch:
        # the batched sweep of 256 uneven cases (its own steady state first)
        out["batch"] = measure_batch(args, args.batch_cases, args.batch_steps, 3, args.batch_budget_s)
    if rank == 0 and args.forward4 and not args.no_forward4:
        # the 4-blade forward-flight rotor: FP32 forms against the plain FP64
        # form over the same steps, the surrogate, 8 batched copies
        out["forward4"] = measure_forward4(args, args.forward_step, K, W)
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_reference(args):
    """Reference arm: the reference's CPU algorithm on the host cores.

    The reference is Fortran and neither machine has a Fortran compiler, so
    the arm runs the oracle -- the C++ FP64 restatement of the reference's
    path, OpenMP over targets as the reference's drivers -- on every host
    core.  It steps the same case through the same steady-state steps as the
    GPU arm's timed window (steps FULL_WAKE_STEP + W + 1 .. + K).  The oracle
    needs tens of minutes for the first 432 steps of this wake, so it starts
    from the state the FP64 GPU solver reaches at step FULL_WAKE_STEP (set-up
    only, outside the timed region: the GPU and the oracle are bit-identical
    step by step in FP64 with the same summation blocks,
    tests/test_gpu_parity_full.py), runs W untimed warm-up steps and K timed
    steps.  The GPU's FP64 form then runs the same W + K steps from the same
    state, and the line reports whether the CT rows agree bit for bit."""
    rank = env_int("RANK", 0)
    if rank != 0:
        return
    from volcanor_gb300 import lib
    K, W = args.steps, args.warmup
    start = FULL_WAKE_STEP
    c = C.rotor_2blade_hover(nt=max(start + W + K + 2, 1440))
    g = lib.Case(c.config, c.geom, precision=lib.PREC_FP64, sum_chunk=256, device=env_int("LOCAL_RANK", 0))
    g.start()
    t_setup = time.perf_counter()
    done = 0
    while done < start:
        n = min(100, start - done)
        g.step(n, with_ct=False)
        done += n
    sim = cpu_handoff(c, g)
    t_setup = time.perf_counter() - t_setup
    threads = os.cpu_count() or 1
    times = []
    for _ in range(W + K):
        t0 = time.perf_counter()
        sim.step(1)
        times.append(time.perf_counter() - t0)
    timed = float(sum(times[W:]))
    val = K / timed
    rows_cpu = sim.ct_hist()[-(W + K):]
    rows_gpu = g.step(W + K)
    same = bool(np.array_equal(rows_cpu, rows_gpu))
    desc = (f"{K} whole timesteps (steps {start + W + 1}-{start + W + K}) after {W} untimed warm-up steps, from the "
            f"FP64 GPU solver's state at step {start}; oracle = C++ FP64 restatement of the reference's path "
            f"(OpenMP over targets, {threads} threads, summation blocks of 256) -- the Fortran reference cannot be "
            "compiled on these machines")
    out = {"impl": "reference", "metric": METRIC, "value": round(val, 4), "unit": "timesteps/s", "n_gpus": 1,
           "steps": K, "warmup": W, "ms_per_step": round(1e3 * timed / K, 2), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (volcanor_gb300/cases.py)",
           "config": {"workload": WORKLOAD, "precision": "fp64 (reference arithmetic)"},
           "cpu_baseline": {"value": round(val, 4), "unit": "timesteps/s", "cores": threads, "kind": "port",
                            "sample": desc},
           "e2e": {"value": round(val, 4), "unit": "timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "ct_rows_bitwise_equal_to_fp64_gpu": same, "setup_s": round(t_setup, 1),
           "timed_s": round(timed, 2)}
    print(json.dumps(out))


def measure_batch(args, n: int, K: int, W: int, budget_s: float = None):
    """Batched sweep: n independent uneven rotor cases (volcanor_gb300/cases.py
    batch_sweep) advanced together; once every case is in its steady state
    each batch step is one CUDA-graph launch.  Returns case-timesteps/s."""
    from volcanor_gb300 import lib
    prec = {"fp32near": lib.PREC_FP32_NEAR64, "fp32": lib.PREC_FP32, "fp64": lib.PREC_FP64}[args.precision]
    steady = 8 * 72 + 2
    cases = C.batch_sweep(n, seed=0, nt=steady + W + 2 * K)
    t0 = time.perf_counter()
    b = lib.Batch([(c.config, c.geom, "") for c in cases], precision=prec)
    b.start()
    done = 0
    while done < steady + W:
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            # the transient (each case's steps launched one by one until
            # every case is steady) takes minutes: a slow box ends the
            # measurement instead of the whole run
            b.close()
            return {"metric": "batched free-wake case-timesteps/s", "value": None, "unit": "case-timesteps/s",
                    "skipped": f"transient not finished within {budget_s:.0f} s of wall time ({done} of "
                               f"{steady + W} steps); python bench.py --workload batch measures it alone"}
        m = min(50, steady + W - done)
        b.step(m, with_ct=False)
        done += m
    warm_s = time.perf_counter() - t0
    l0 = lib.launch_count()
    with ClockSampler(env_int("LOCAL_RANK", 0)) as clk:
        rows = b.step(K)
        ms = b.last_step_ms()
    launches = lib.launch_count() - l0
    value = n * K / (ms / 1e3)
    # e2e: single batch steps through the public API (frames in, CT rows out)
    t1 = time.perf_counter()
    for _ in range(K):
        b.step(1)
    e2e = n * K / (time.perf_counter() - t1)
    b.close()
    return {"metric": "batched free-wake case-timesteps/s", "value": round(value, 2), "unit": "case-timesteps/s",
            "steps": K, "warmup": W, "ms_per_step": round(ms / K, 4),
            "workload": f"{n} independent rotor cases: 2-4 blades, 24-400 rings, collective 2-12 deg, advance ratio "
                        "0-0.3, wakes of 1-8 revolutions (5k-120k filaments), steady state, one CUDA-graph launch "
                        "per batch step", "precision": args.precision,
            "e2e": {"value": round(e2e, 2), "unit": "case-timesteps/s", "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": n * 80},
            "gpu_launches": int(launches), "graph_launches_per_step": 1, "warmup_wall_s": round(warm_s, 1),
            "clocks": clk.summary(), "ct_finite": bool(np.all(np.isfinite(rows)))}


def run_batch(args):
    """The batched sweep alone (--workload batch)."""
    r = measure_batch(args, args.batch_cases, args.steps, args.warmup)
    out = {"metric": r.pop("metric"), "value": r.pop("value"), "unit": r.pop("unit"), "n_gpus": 1,
           "steps": r.pop("steps"), "warmup": r.pop("warmup"), "ms_per_step": r.pop("ms_per_step"),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
           "data": f"synthetic ({args.batch_cases} seeded uneven rotor cases, volcanor_gb300/cases.py batch_sweep)",
           "config": {"workload": r.pop("workload"), "precision": r.pop("precision")}}
    out.update(r)
    print(json.dumps(out))


def measure_forward4(args, S: int, K: int, W: int, batched: bool = True):
    """4-blade rotor in forward flight (R = 2 m, c = 0.12 m, -8 deg twist,
    theta0 = 10 deg, mu = 0.1, shaft tilt -4 deg, 1 x 32 rings per blade,
    dt = 5 deg, 1 rev of near wake, untruncated far wake), K timed steps after
    S + W steps from the start: the FP32 + FP64 near-field form, the plain
    FP64 form from the FP32 form's state at the window start (its CT error
    over the window in SYNC-step segments re-started from the FP32 state), the
    FP32 form with the learned surrogate of the old far wake, and 8 batched
    copies of the FP32 form."""
    import tempfile
    from volcanor_gb300 import lib
    nt = S + W + K
    SYNC = 20
    tmp = tempfile.TemporaryDirectory()
    cdir = Path(tmp.name) / "case"
    c = C.rotor_4blade_forward(nt=nt)
    c.write(cdir)

    def make(prec, surr=None):
        g = lib.Case.from_case_dir(cdir, precision=prec)
        if surr is not None:
            g.set_surrogate(**surr)
        g.start()
        return g

    def advance(g, n):
        done = 0
        while done < n:
            m = min(100, n - done)
            g.step(m, with_ct=False)
            done += m

    res = {}
    g = make(lib.PREC_FP32_NEAR64)
    advance(g, S + W)
    ck = Path(tmp.name) / "window.ckpt"
    g.checkpoint_save(ck)
    rows32 = g.step(K)
    ms = g.last_step_ms()
    res["fp32near"] = {"timesteps_per_s": round(K / (ms / 1e3), 3), "ms_per_step": round(ms / K, 3)}
    # the plain FP64 form over the same steps from the same state
    f = lib.Case.from_case_dir(cdir, precision=lib.PREC_FP64)
    f.checkpoint_load(ck)
    rows64 = f.step(K)
    ms64 = f.last_step_ms()
    res["fp64"] = {"timesteps_per_s": round(K / (ms64 / 1e3), 3), "ms_per_step": round(ms64 / K, 3)}
    seg = []
    g.checkpoint_load(ck)
    ckj = Path(tmp.name) / "seg.ckpt"
    for j in range(0, K, SYNC):
        n = min(SYNC, K - j)
        g.checkpoint_save(ckj)
        a = g.step(n)[:, 1]
        f.checkpoint_load(ckj)
        b = f.step(n)[:, 1]
        seg.append(float(np.max(np.abs(a - b) / np.abs(b))))
    res["fp32near"]["ct_max_rel_err_vs_fp64_timed_window"] = max(seg)
    res["fp32near"]["ct_max_rel_err_unsynced"] = float(np.max(np.abs(rows32[:, 1] - rows64[:, 1]) /
                                                              np.abs(rows64[:, 1])))
    g.close()
    f.close()
    # with the learned surrogate (its own run from the start: it collects its
    # training data from the solver)
    h = make(lib.PREC_FP32_NEAR64, {})
    advance(h, S + W)
    rows_s = h.step(K)
    ms = h.last_step_ms()
    res["fp32near_surrogate"] = {"timesteps_per_s": round(K / (ms / 1e3), 3), "ms_per_step": round(ms / K, 3),
                                 "surrogate": h.surrogate_stats()}
    h.close()
    if batched:
        b = lib.Batch([(c.config, c.geom, str(cdir))] * 8, precision=lib.PREC_FP32_NEAR64)
        b.start()
        done = 0
        while done < S + W:
            m = min(100, S + W - done)
            b.step(m, with_ct=False)
            done += m
        b.step(K, with_ct=False)
        ms = b.last_step_ms()
        res["fp32near_batched_x8"] = {"case_timesteps_per_s": round(8 * K / (ms / 1e3), 3)}
        b.close()
    base = res["fp64"]["timesteps_per_s"]
    res["speedup_vs_fp64"] = {k: round((v.get("timesteps_per_s") or v.get("case_timesteps_per_s")) / base, 1)
                              for k, v in res.items() if isinstance(v, dict) and k != "fp64"}
    res["window"] = [S + W + 1, S + W + K]
    res["sync_every_steps"] = SYNC
    tmp.cleanup()
    return res


def run_forward4(args):
    """The 4-blade forward-flight workload alone (--workload forward4)."""
    K, W = args.steps, args.warmup
    res = measure_forward4(args, args.forward_step, K, W)
    out = {"metric": "free-wake timesteps/s, 4-blade forward-flight rotor", "unit": "timesteps/s",
           "value": res["fp32near"]["timesteps_per_s"], "n_gpus": 1, "steps": K, "warmup": W,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32near",
           "data": "synthetic (case files generated by volcanor_gb300/cases.py rotor_4blade_forward)",
           "config": {"workload": f"4-blade forward flight, steps {res['window'][0]}..{res['window'][1]} of an "
                                  "untruncated wake"},
           "forms": res}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32near", choices=["fp32near", "fp32", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-kernel", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--kernel-reps", type=int, default=3)
    ap.add_argument("--kernel-only", action="store_true",
                    help="only the isolated ring kernel (for profiling); prints its JSON")
    ap.add_argument("--kernel-m", type=int, default=1 << 20)
    ap.add_argument("--forward-step", type=int, default=720)
    ap.add_argument("--workload", default="hover2", choices=["hover2", "batch", "forward4"],
                    help="hover2: the headline 2-blade hover case; batch: 256 uneven cases in one graph launch")
    ap.add_argument("--batch-cases", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=10, help="timed steps of the batch key")
    # the batched sweep's transient takes ~3 min (581 steps of 256 cases):
    # a key of the default line with a wall-clock budget; the forward-flight
    # rotor is an opt-in key (or its own --workload)
    ap.add_argument("--batch-budget-s", type=float, default=240.0,
                    help="wall time the batch key's transient may take before the key is skipped")
    ap.add_argument("--no-batch", action="store_true", help="leave the batched sweep out of the line")
    ap.add_argument("--forward4", action="store_true", help="add the 4-blade forward-flight key")
    ap.add_argument("--no-forward4", action="store_true", help="(default) no forward-flight key")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.kernel_only:
        from volcanor_gb300 import lib
        kp = {"fp32near": lib.PREC_FP32_NEAR64, "fp32": lib.PREC_FP32, "fp64": lib.PREC_FP64}[args.precision]
        print(json.dumps(run_kernel_cfg3(kp, reps=args.kernel_reps, M=args.kernel_m)))
        return
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "forward4":
        run_forward4(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

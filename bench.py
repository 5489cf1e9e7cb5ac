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
       all cores), a bounded sample of the same workload per step.
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


def cpu_sample(case_gpu, seconds: float = 12.0, max_targets: int = 4096):
    """Oracle (C++ restatement, OpenMP all cores) on a bounded sample of the
    steady-state wake: sampled wake-node targets x every near-wake ring of the
    GPU state.  Returns (ring pairs/s, threads, description)."""
    from oracle import oracle as O
    nb = case_gpu.geti("nb")
    corners, rvc, gam, nodes = [], [], [], []
    for b in range(1, nb + 1):
        c = case_gpu.get("waN", b).reshape(-1, 4, 3)
        corners.append(c)
        rvc.append(case_gpu.get("waN_rvc", b).reshape(-1, 4))
        gam.append(case_gpu.get("waN_gam", b))
        nodes.append(c[:, 1])
    corners, rvc, gam = np.concatenate(corners), np.concatenate(rvc), np.concatenate(gam)
    nodes = np.concatenate(nodes)
    rng = np.random.default_rng(0)
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    m = 64
    t = 0.0
    while True:
        P = nodes[rng.choice(len(nodes), size=min(m, len(nodes)), replace=False)]
        t0 = time.perf_counter()
        O.vind_rings(corners, rvc, gam, P)
        t = time.perf_counter() - t0
        if t > seconds / 4 or m >= max_targets:
            break
        m *= 2
    pairs = float(P.shape[0]) * corners.shape[0]
    desc = (f"{P.shape[0]} wake-node targets x {corners.shape[0]} near-wake rings of the steady-state wake "
            f"({pairs:.3g} ring pairs, {t:.2f} s)")
    return pairs / t, threads, desc


def pairs_per_step(case_gpu):
    """Ring-equivalent pairs (4 filament pairs = 1 ring pair) of one steady-state
    step: two wake-node evaluations (wing + wake sources) and the
    collocation-point evaluation (wake sources)."""
    g = case_gpu.geti
    nb, nc, ns, NW, NF, nbc = g("nb"), g("nc"), g("ns"), g("nNwake"), g("nFwake"), g("nbConvect")
    m_nodes = nbc * (NW * (ns + 1) + NF)
    src_wake = nb * NW * ns + nb * (ns + NF) / 4.0
    src_all = nb * nc * ns + src_wake
    return 2.0 * m_nodes * src_all + nbc * nc * ns * src_wake


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
    case = lib.Case(c.config, c.geom, precision=prec)
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("CUDA_VISIBLE_DEVICES", ""))
    case.start()
    # reach the steady state, then W warm-up steps
    done = 0
    while done < FULL_WAKE_STEP + W:
        n = min(100, FULL_WAKE_STEP + W - done)
        case.step(n, with_ct=False)
        done += n
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        l0 = lib.launch_count()
        t0 = time.perf_counter()
        rows = case.step(K)
        launches = lib.launch_count() - l0
        wall = time.perf_counter() - t0
        dev_ms = case.last_step_ms()
    if dist:
        import torch
        t = torch.tensor([dev_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms = float(t.item())
    value = world * K / (dev_ms / 1e3)
    # e2e: one public-API call per step with host buffers
    e2e_steps = K
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        case.step(1)
    e2e_wall = time.perf_counter() - t0
    e2e = world * e2e_steps / e2e_wall
    frame_doubles = None
    try:
        nb, nc, ns = case.geti("nb"), case.geti("nc"), case.geti("ns")
        frame_doubles = nb * nc * ns * 27 + nb * ns * 12 + nb * 9 + 10 + 9 * (nb - 1)
    except Exception:
        pass
    # roofline of the dominant kernel on the live steady-state state
    with nvtx_range("profile_eval"):
        ms_l, rp, fp = case.profile_eval(20)
    near_pairs = case.geti("nearPairs") if prec == lib.PREC_FP32_NEAR64 else 0
    node_chunks = case.geti("nodeChunks")
    flops = RING_FLOP * rp + FIL_FLOP * fp
    achieved = flops / (ms_l / 1e3) / 1e12
    pk = peaks()
    sm_max = pk.get("sm_max_mhz", 2070.0)
    sm_count = lib.device_info(local)[0]
    fp32_peak = sm_count * 128 * 2 * sm_max * 1e6 / 1e12
    clocks = clk.summary()
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
                     "near_pairs_per_launch": near_pairs, "chunks": node_chunks,
                     "peak_note": "nominal FP32 CUDA-core peak (SMs x 128 lanes x 2 x max SM clock); "
                                  "MEASURED_PEAKS.json has no FP32 figure"},
        "clocks": clocks,
        "ct_last": float(rows[-1, 1]),
    }
    out["pairs_per_s"] = round(rp / (ms_l / 1e3), 1)
    if not args.no_kernel:
        kp = {"fp32near": lib.PREC_FP32_NEAR64, "fp32": lib.PREC_FP32, "fp64": lib.PREC_FP32_NEAR64}[args.precision]
        k3 = run_kernel_cfg3(kp, reps=args.kernel_reps)
        k3["frac_of_fp32_peak"] = round(k3["tflops"] / fp32_peak, 4)
        k3["workload"] = "isolated kernel: 2^20 targets x 2^18 rings (U[0,1]^3, edges U(0.005,0.05), core 0.002)"
        out["kernel_rings"] = k3
    if rank == 0 and not args.no_cpu:
        try:
            rate, threads, desc = cpu_sample(case, seconds=args.cpu_seconds)
            eq = pairs_per_step(case)
            out["cpu_baseline"] = {"value": round(rate / eq, 4), "unit": "timesteps/s", "cores": threads,
                                   "kind": "port", "sample": desc + f"; converted at {eq:.4g} ring pairs per step"}
        except Exception as e:  # the baseline is reported, never required
            out["cpu_baseline"] = {"value": None, "unit": "timesteps/s", "cores": None, "kind": "port",
                                   "sample": f"failed: {e}"}
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def helix_wake(nb: int, ns: int, nw: int, radius: float, rootcut: float, omega: float, dt: float,
               core: float, seed: int = 0):
    """Near-wake rings of a prescribed helical hover wake with the case's node
    counts (nb blades x nw rows x ns rings): node (i, j) of blade b at radius
    r_j, azimuth 2 pi b / nb - omega dt i, descending at the momentum-theory
    induced velocity.  The FP64 filament kernel's cost does not depend on the
    positions, so this stands in for the solver's wake in CPU timing."""
    rng = np.random.default_rng(seed)
    r = np.linspace(rootcut * radius, radius, ns + 1)
    vi = omega * radius * np.sqrt(0.0035 / 2.0)
    corners = []
    for b in range(nb):
        i = np.arange(nw + 1)[:, None]
        psi = 2.0 * np.pi * b / nb - omega * dt * i
        x, y = r[None, :] * np.cos(psi), r[None, :] * np.sin(psi)
        z = np.broadcast_to(-vi * dt * i, x.shape)
        nodes = np.stack([x, y, z], -1)  # [row][station]
        c = np.stack([nodes[:-1, :-1], nodes[1:, :-1], nodes[1:, 1:], nodes[:-1, 1:]], 2)  # [row][ring][4][3]
        corners.append(c.reshape(-1, 4, 3))
    corners = np.concatenate(corners)
    rvc = np.full((corners.shape[0], 4), core)
    gam = rng.normal(0.0, 0.05, corners.shape[0])
    nodes = corners[:, 1]
    return corners, rvc, gam, nodes


def oracle_pairs_per_step(sim):
    """pairs_per_step from the oracle's case dimensions."""
    g = sim.geti
    nb, nc, ns, NW, NF, nbc = g("nb"), g("nc"), g("ns"), g("nNwake"), g("nFwake"), g("nbConvect")
    m_nodes = nbc * (NW * (ns + 1) + NF)
    src_wake = nb * NW * ns + nb * (ns + NF) / 4.0
    src_all = nb * nc * ns + src_wake
    return 2.0 * m_nodes * src_all + nbc * nc * ns * src_wake


def run_reference(args):
    """Reference arm: the reference algorithm on the host cores, no GPU.  The
    reference is Fortran and no Fortran compiler exists here, so this times
    the oracle (the C++ FP64 restatement, OpenMP over targets like the
    reference): each "step" is a bounded sample -- sampled wake-node targets x
    every near-wake ring of a steady-state-sized helical wake -- converted to
    timesteps/s by the ring pairs of one steady-state step of the case."""
    rank = env_int("RANK", 0)
    if rank != 0:
        return
    import tempfile
    from oracle import oracle as O
    K, W = args.steps, args.warmup
    c = C.rotor_2blade_hover(nt=1440)
    with tempfile.TemporaryDirectory() as d:
        c.write(d)
        sim = O.Sim.from_case_dir(d)
    eq = oracle_pairs_per_step(sim)
    nb, ns, NW = sim.geti("nb"), sim.geti("ns"), sim.geti("nNwake")
    corners, rvc, gam, nodes = helix_wake(nb, ns, NW, 1.0, 0.2, 100.0, 5.0 * np.pi / 180.0 / 100.0, 0.004)
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    rng = np.random.default_rng(0)
    per_step = args.cpu_seconds / max(1, W + K)
    # size the sample once: doubling target counts until one call takes a step's share
    m = 64
    while True:
        P = nodes[rng.choice(len(nodes), size=min(m, len(nodes)), replace=False)]
        t0 = time.perf_counter()
        O.vind_rings(corners, rvc, gam, P)
        t = time.perf_counter() - t0
        if t > per_step / 2 or m >= 4096:
            break
        m *= 2
    rates = []
    for i in range(W + K):
        P = nodes[rng.choice(len(nodes), size=P.shape[0], replace=False)]
        t0 = time.perf_counter()
        O.vind_rings(corners, rvc, gam, P)
        t = time.perf_counter() - t0
        if i >= W:
            rates.append(P.shape[0] * corners.shape[0] / t)
    val = float(np.mean(rates)) / eq
    desc = (f"{P.shape[0]} wake-node targets x {corners.shape[0]} near-wake rings of a helical wake with the case's "
            f"node counts, {K} timed samples after {W} warm-up; oracle (C++ FP64 restatement, not the Fortran "
            f"reference: no Fortran compiler); converted at {eq:.4g} ring pairs per step")
    out = {"impl": "reference", "metric": METRIC, "value": round(val, 4), "unit": "timesteps/s", "n_gpus": 1,
           "steps": K, "warmup": W, "ms_per_step": round(1e3 / val, 3), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": {"workload": WORKLOAD},
           "cpu_baseline": {"value": round(val, 4), "unit": "timesteps/s", "cores": threads, "kind": "port",
                            "sample": desc},
           "e2e": {"value": round(val, 4), "unit": "timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32near", choices=["fp32near", "fp32", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-kernel", action="store_true")
    ap.add_argument("--kernel-reps", type=int, default=3)
    ap.add_argument("--kernel-only", action="store_true",
                    help="only the isolated ring kernel (for profiling); prints its JSON")
    ap.add_argument("--kernel-m", type=int, default=1 << 20)
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
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

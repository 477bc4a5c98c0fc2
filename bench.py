"""Throughput of the explicit right-hand-side path: point-updates/s per RK stage.

Workload (default): 2-D compressible Euler, gamma 1.4, on [0,1]^2, jittered lattice h = 1e-3 (±0.25h), about 1.0M
interior particles plus ghosts; four-quadrant Riemann initial state split at (0.5, 0.5); transmissive (outflow)
boundaries; MUSCL order 2 with the MLS divergence fit of order 2; MOOD (EPD1, MOODu1 with delta = 1e-4 h^2);
Rusanov flux; SSP-RK3; dt = 0.4 x the CFL step at the initial state. Synthetic, seeded inputs (no dataset).

`value` is the FP32 bulk path with the learned troubled-point predictor attached (the headline; the plain FP32
path is `fp32_plain`), measured with the state resident in HBM; `e2e` is the same metric through the C ABI with
host buffers (state uploaded from pinned memory and downloaded every step); `fp64_plain` is the plain FP64 path on
the same cloud; `accuracy_vs_finer_fp64` compares the density L1 errors of the three against an FP64 run at h/2.
`roofline` rates the flux pass (and, under `roofline.gather`, the reconstruction pre-pass) against the measured HBM
copy peak. Every context is tuned by `hcc_autotune` before its timed region (`--no-autotune`: default shapes).
`euler3d_blast_8M` and `ensemble` add the 3-D blast (with its own equal-L1 study at 1.0M) and the 512-cloud
batched ensemble. `cpu_baseline` times the CPU oracle (the C++ restatement of the reference's CPU path) on a
bounded sample of the same workload. `--impl reference` runs only that CPU path.

Launch: python bench.py [--gpus N --steps K --warmup W]; for N > 1 under torch.distributed.run (one rank per GPU,
independent replicas: the path does not shard).
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "hypercloudcore.jl_gb300"
METRIC = "point-updates/s per RK stage, FP32+learned vs plain FP64 on 1 GB300 at equal L1"
STAGES = 3
HOST_DRIVEN = False     # --host-driven: steps without the step graph (e.g. for kernel profilers)
AUTOTUNE = True         # --no-autotune: keep the default launch shapes (hcc_autotune picks them otherwise)


def _load(name, path, pkg_dir=None):
    if name in sys.modules:
        return sys.modules[name]
    kw = {"submodule_search_locations": [str(pkg_dir)]} if pkg_dir else {}
    spec = importlib.util.spec_from_file_location(name, path, **kw)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def package():
    return _load("hcc_gb300", PKG / "__init__.py", PKG)


# --------------------------------------------------------------------------------------------- workload
WORKLOADS = {
    # name: (dim, h, description)
    "euler2d_quadrant_1M": (2, 1e-3, "2-D Euler quadrant Riemann, h=1e-3 (1.0M interior), MUSCL2+MOOD, SSP-RK3"),
    "euler2d_quadrant_250k": (2, 2e-3, "2-D Euler quadrant Riemann, h=2e-3 (250k interior), MUSCL2+MOOD, SSP-RK3"),
    "euler3d_blast_8M": (3, 1 / 200, "3-D Euler spherical blast, h=1/200 (8.0M interior), MUSCL2+MOOD, SSP-RK3"),
    "euler3d_blast_1M": (3, 1 / 100, "3-D Euler spherical blast, h=1/100 (1.0M interior), MUSCL2+MOOD, SSP-RK3"),
}


def quadrant_state(cloud, gamma=1.4):
    x, y = cloud.pos[:, 0], cloud.pos[:, 1]
    vals = {"NE": (1.5, 0.0, 0.0, 1.5), "NW": (0.5323, 1.206, 0.0, 0.3),
            "SW": (0.138, 1.206, 1.206, 0.029), "SE": (0.5323, 0.0, 1.206, 0.3)}
    rho, u, v, p = (np.empty(cloud.n) for _ in range(4))
    for key, (r0, u0, v0, p0) in vals.items():
        sel = ((x >= 0.5) if key[1] == "E" else (x < 0.5)) & ((y >= 0.5) if key[0] == "N" else (y < 0.5))
        rho[sel], u[sel], v[sel], p[sel] = r0, u0, v0, p0
    E = p / (gamma - 1) + 0.5 * rho * (u * u + v * v)
    return np.ascontiguousarray(np.stack([rho, rho * u, rho * v, E], axis=1))


def blast_state(cloud, gamma=1.4):
    """Spherical blast: rho = 1, p = 1 for r < 0.2 about the centre, else rho = 0.125, p = 0.1; zero velocity."""
    r2 = ((cloud.pos - 0.5) ** 2).sum(axis=1)
    inside = r2 < 0.04
    rho = np.where(inside, 1.0, 0.125)
    p = np.where(inside, 1.0, 0.1)
    D = cloud.pos.shape[1]
    return np.ascontiguousarray(np.column_stack([rho] + [np.zeros_like(rho)] * D + [p / (gamma - 1)]))


def make_workload(hcc, name):
    D, h, _ = WORKLOADS[name]
    cloud = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h, 2.5 * h, jitter=0.25 * h, seed=42)
    U0 = quadrant_state(cloud) if D == 2 else blast_state(cloud)
    return cloud, U0, h


def make_cfg(hcc, cloud, h, precision):
    """MUSCL order 2 with the divergence fit of order 2, MOOD (EPD1, MOODu1(1e-4 h^D)), Rusanov, SSP-RK3,
    transmissive boundaries on every wall."""
    D = cloud.pos.shape[1]
    return hcc.make_config(hcc.Euler(D, 1.4), cloud, scheme=hcc.MUSCL(2, 2),
                           mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h ** D)), tableau="RK3_SSP",
                           bc_map={t: hcc.BC_OUTFLOW for t in range(1, 2 * D + 1)}, precision=precision)


# --------------------------------------------------------------------------------------------- helpers
class ClockSampler:
    """SM clocks and clock-event (throttle) reasons sampled while the timed region runs: NVML through ctypes every
    millisecond (a timed region of ten 1-ms steps still gets samples), else `nvidia-smi -lms 200`. Reads only."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason* bits
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}

    def __init__(self, gpu_index=0, period_s=0.001):
        self.gpu = gpu_index
        self.period = period_s
        self.proc = None
        self.lines = []
        self.samples = []           # (sm_mhz, max_mhz, reason bits) from NVML
        self.nvml = None
        self.stop = threading.Event()

    def _open_nvml(self):
        import ctypes as C
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
        except OSError:
            return None
        if lib.nvmlInit_v2() != 0:
            return None
        dev = C.c_void_p()
        bus = self._pci_bus_id()
        if bus is not None and lib.nvmlDeviceGetHandleByPciBusId_v2(C.c_char_p(bus.encode()), C.byref(dev)) == 0:
            pass
        elif lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.gpu), C.byref(dev)) != 0:
            lib.nvmlShutdown()
            return None
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons", None)
        if reasons is None:
            lib.nvmlShutdown()
            return None
        return lib, dev, reasons

    def _pci_bus_id(self):
        """The CUDA device's PCI address in NVML's form (NVML numbers GPUs without CUDA_VISIBLE_DEVICES)."""
        try:
            import torch
            p = torch.cuda.get_device_properties(self.gpu)
            return f"{p.pci_domain_id:08X}:{p.pci_bus_id:02X}:{p.pci_device_id:02X}.0"
        except Exception:
            return None

    def _poll(self):
        import ctypes as C
        lib, dev, reasons = self.nvml
        cur, mx, bits = C.c_uint(), C.c_uint(), C.c_ulonglong()
        while True:
            ok = lib.nvmlDeviceGetClockInfo(dev, 1, C.byref(cur)) == 0          # NVML_CLOCK_SM
            ok = ok and lib.nvmlDeviceGetMaxClockInfo(dev, 1, C.byref(mx)) == 0
            ok = ok and reasons(dev, C.byref(bits)) == 0
            if ok:
                self.samples.append((float(cur.value), float(mx.value), int(bits.value)))
            if self.stop.wait(self.period):
                break

    def __enter__(self):
        self.nvml = self._open_nvml()
        if self.nvml:
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
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

    def __exit__(self, *exc):
        if self.nvml:
            self.stop.set()
            self.t.join(timeout=2)
            self.nvml[0].nvmlShutdown()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        for cur, m, bits in self.samples:
            sm.append(cur)
            mx = m
            reasons.update(nm for nm, b in self.BITS.items() if bits & b)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvml" if self.samples else "nvidia-smi"}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def recorded_traffic():
    """Per-point-stage DRAM bytes of the flux kernel from the committed ncu summary (profiles/traffic.txt)."""
    p = ROOT / "profiles" / "traffic.txt"
    out = {}
    if p.exists():
        for ln in p.read_text().splitlines():
            ln = ln.strip()
            if ln and not ln.startswith("#"):
                k, v = ln.split()[:2]
                out[k] = float(v)
    return out


def algorithmic_bytes(K, D, M, Br, Bd, s):
    """Bytes per point and RK stage that the two passes must move (the model of the measurement plan):
    flux pass 4K + 8D + 8 Bd^2 + s M (5 + Br); gather pass 4K + 8D + 8 Br^2 + s M (1 + Br)."""
    flux = 4 * K + 8 * D + 8 * Bd * Bd + s * M * (5 + Br)
    gather = 4 * K + 8 * D + 8 * Br * Br + s * M * (1 + Br)
    return flux, gather


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------------------------- GPU arm
def time_device_steps(hcc, ctx, dt, steps, world):
    """K steps with the state resident in HBM, CUDA events on the context's stream, max over ranks."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    launches0 = ctx.counters()["kernel_launches_total"]
    barrier(world)
    ctx.synchronize()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        ctx.step(0.0, dt)
    e1.record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    launches = ctx.counters()["kernel_launches_total"] - launches0
    return reduce_max(ms, world), launches


def time_e2e(hcc, ctx, U_host, dt, steps, world, f32):
    """The same steps through the C ABI with host buffers: upload (pinned) -> step -> download, every step."""
    import torch
    dtype = torch.float32 if f32 else torch.float64
    pinned = torch.empty(U_host.shape, dtype=dtype, pin_memory=True)
    pinned.copy_(torch.from_numpy(U_host.astype(np.float32 if f32 else np.float64)))
    host = pinned.numpy()
    out = torch.empty(U_host.shape, dtype=dtype, pin_memory=True).numpy()
    barrier(world)
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.upload_state(host)
        ctx.step(0.0, dt)
        ctx.download_state(out=out)
    ctx.synchronize()
    el = time.perf_counter() - t0
    barrier(world)
    return reduce_max(el, world), host.nbytes, out.nbytes


def load_predictor(hcc):
    """The troubled-point predictor shipped with the package (train_predictor.py recipe), or None."""
    learned = sys.modules["hcc_gb300.learned"]
    path = learned.default_weights_path()
    if not path.exists():
        return None
    pred = hcc.TroubledPointPredictor(capacity=16)
    pred.load(path)
    return pred


PREDICTOR_THRESHOLD = 0.9
# the 2-D-trained network on 3-D stencils: a higher threshold keeps the density L1 error within 1.1x of FP64's
# (1.095x at 0.95 against 1.105x at 0.9 on the 1.0M blast after 10 steps)
PREDICTOR_THRESHOLD_3D = 0.95


def measure(hcc, cloud, U0, h, prec, steps, warmup, world, local, e2e=True, acc_dt=None, acc_steps=0,
            predictor=None, threshold=None):
    """One precision on one workload: K device-timed steps (the step graph, no profiling), the same K steps again
    with per-kernel CUDA events (host-driven step) for the roofline, the end-to-end C-ABI leg, and — when asked —
    `acc_steps` steps from the initial state with a fixed dt whose final density is returned for the L1 check.
    With a predictor, every step pre-lowers the particles it predicts troubled (MOOD still judges all)."""
    f32 = prec == "fp32"
    ctx = hcc.Context(make_cfg(hcc, cloud, h, prec))
    if predictor is not None:
        ctx.set_predictor(predictor, PREDICTOR_THRESHOLD if threshold is None else threshold)
    if HOST_DRIVEN:
        ctx.set_step_graphs(False)
    ctx.upload_cloud(cloud)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    U_in = U0.astype(np.float32) if f32 else U0
    ctx.upload_state(U_in)
    dt = 0.4 * ctx.time_step()
    for _ in range(warmup):
        ctx.step(0.0, dt)
    ctx.upload_state(U_in)
    tune = ctx.autotune(dt, steps=3) if AUTOTUNE else None
    with ClockSampler(local) as clk:
        ms, launches = time_device_steps(hcc, ctx, dt, steps, world)
    cnt = ctx.counters()
    ctx.upload_state(U_in)
    ctx.set_profiling(True)
    ctx.kernel_times(reset=True)
    for _ in range(steps):
        ctx.step(0.0, dt)
    ctx.synchronize()
    ctx.set_profiling(False)
    kt = ctx.kernel_times(reset=True)
    out = {"ms": ms, "launches": launches, "kt": kt, "clocks": clk.summary(), "counters": cnt, "dt": dt,
           "tuning": tune}
    if e2e:
        out["e2e_s"], out["h2d"], out["d2h"] = time_e2e(hcc, ctx, U0, dt, steps, world, f32)
    if acc_steps:
        ctx.upload_state(U_in)
        for _ in range(acc_steps):
            ctx.step(0.0, dt if acc_dt is None else acc_dt)
        out["rho"] = ctx.download_state(dtype=np.float64)[:, 0].copy()
    ctx.close()
    return out


def rel_l1(a, b, sel):
    return float(np.abs(a[sel] - b[sel]).sum() / np.abs(b[sel]).sum())


def fine_reference(hcc, cloud, h, dt, steps):
    """Density of the plain FP64 path on the same problem at spacing h/2 after 2*steps steps of dt/2 (the same
    final time), sampled at the particles of `cloud` (nearest fine particle): the reference of the L1 errors."""
    from scipy.spatial import cKDTree
    D = cloud.pos.shape[1]
    fine = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h / 2, 2.5 * h / 2, jitter=0.25 * h / 2, seed=42)
    ctx = hcc.Context(make_cfg(hcc, fine, h / 2, "fp64"))
    ctx.upload_cloud(fine)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    ctx.upload_state(quadrant_state(fine) if D == 2 else blast_state(fine))
    for _ in range(2 * steps):
        ctx.step(0.0, dt / 2)
    rho = ctx.download_state()[:, 0].copy()
    ctx.close()
    _, idx = cKDTree(fine.pos).query(cloud.pos)
    return rho[idx]


def run_3d(hcc, args, world, local):
    """The 3-D Euler blast at 8.0M interior particles (K ~ 67): FP32 bulk and FP64 plain step rates and the FP32
    density's relative L1 distance from the FP64 run after the same steps; and the density L1 errors of FP64, FP32
    and FP32 + predictor at 1.0M interior against the FP64 path at h/2."""
    name = "euler3d_blast_8M"
    cloud, U0, h = make_workload(hcc, name)
    n_int = cloud.n_interior
    steps32, steps64, acc = max(3, min(args.steps, 10)), 2, 5
    r32 = measure(hcc, cloud, U0, h, "fp32", steps32, 2, world, local, e2e=False)
    dt = r32["dt"]
    r32a = measure(hcc, cloud, U0, h, "fp32", 1, 0, world, local, e2e=False, acc_dt=dt, acc_steps=acc)
    r64 = measure(hcc, cloud, U0, h, "fp64", steps64, 1, world, local, e2e=False, acc_dt=dt, acc_steps=acc)
    inner = cloud.is_boundary == 0
    K = r32["counters"]["total_neighbours"] / max(cloud.n, 1)
    kt = r32["kt"]
    learned = {}
    predictor = None if args.no_learned else load_predictor(hcc)
    if predictor is not None:
        # the network trained on 2-D runs, applied as-is to the 3-D stencils (MOOD still judges every particle)
        rl = measure(hcc, cloud, U0, h, "fp32", steps32, 2, world, local, e2e=False, predictor=predictor,
                     threshold=PREDICTOR_THRESHOLD_3D)
        rla = measure(hcc, cloud, U0, h, "fp32", 1, 0, world, local, e2e=False, acc_dt=dt, acc_steps=acc,
                      predictor=predictor, threshold=PREDICTOR_THRESHOLD_3D)
        learned = {"fp32_learned": {"threshold": PREDICTOR_THRESHOLD_3D,
                                    "value": n_int * STAGES * steps32 * world / (rl["ms"] / 1e3),
                                    "ms_per_step": rl["ms"] / steps32,
                                    "mood_iterations_last_step": rl["counters"]["mood_iterations"],
                                    "predicted_last_step": rl["counters"]["predicted"], "clocks": rl["clocks"]},
                   "l1_density_learned_vs_fp64": {"value": rel_l1(rla["rho"], r64["rho"], inner), "steps": acc,
                                                  "dt": dt}}
    accuracy = {}
    if not args.no_reference_solution:
        # equal-L1 check in 3-D: the blast at h = 1/100 (1.0M interior) in FP64, FP32 and FP32 + predictor against
        # the FP64 path at h/2 (8.0M interior, twice the steps at dt/2)
        c1, u1, h1 = make_workload(hcc, "euler3d_blast_1M")
        steps1 = 10
        a64 = measure(hcc, c1, u1, h1, "fp64", 1, 0, world, local, e2e=False, acc_steps=steps1)
        dt1 = a64["dt"]
        a32 = measure(hcc, c1, u1, h1, "fp32", 1, 0, world, local, e2e=False, acc_dt=dt1, acc_steps=steps1)
        ref = fine_reference(hcc, c1, h1, dt1, steps1)
        in1 = c1.is_boundary == 0
        accuracy = {"reference": "FP64 plain at h/2 (8x the particles), 2x the steps at dt/2, nearest fine particle",
                    "workload": "euler3d_blast_1M", "steps": steps1, "dt": dt1,
                    "l1_fp64": rel_l1(a64["rho"], ref, in1), "l1_fp32": rel_l1(a32["rho"], ref, in1)}
        accuracy["fp32_over_fp64"] = accuracy["l1_fp32"] / accuracy["l1_fp64"]
        if predictor is not None:
            al = measure(hcc, c1, u1, h1, "fp32", 1, 0, world, local, e2e=False, acc_dt=dt1, acc_steps=steps1,
                         predictor=predictor, threshold=PREDICTOR_THRESHOLD_3D)
            accuracy["l1_fp32_learned"] = rel_l1(al["rho"], ref, in1)
            accuracy["learned_over_fp64"] = accuracy["l1_fp32_learned"] / accuracy["l1_fp64"]
        accuracy = {"accuracy_vs_finer_fp64": accuracy}
    return {"workload": name, "description": WORKLOADS[name][2], "n_particles": cloud.n, "n_interior": n_int,
            "mean_neighbours": K,
            "fp32": {"value": n_int * STAGES * steps32 * world / (r32["ms"] / 1e3), "ms_per_step": r32["ms"] / steps32,
                     "flux_ms_per_launch": kt["flux_ms"] / max(kt["flux_launches"], 1),
                     "gather_ms_per_launch": kt["gather_ms"] / max(kt["gather_launches"], 1),
                     "mood_iterations_last_step": r32["counters"]["mood_iterations"], "clocks": r32["clocks"]},
            "fp64_plain": {"value": n_int * STAGES * steps64 * world / (r64["ms"] / 1e3),
                           "ms_per_step": r64["ms"] / steps64, "clocks": r64["clocks"]},
            "l1_density_fp32_vs_fp64": {"value": rel_l1(r32a["rho"], r64["rho"], inner), "steps": acc, "dt": dt},
            **learned, **accuracy}


def run_ensemble(hcc, args, world, local):
    """Batched ensemble: `args.ensemble_clouds` independent 2-D clouds (default 512) with log-uniform node counts in
    [4k, 256k] (seeded), one spacing h = 1/256, jittered lattices with transmissive walls. Even clouds: Euler
    (gamma 1.4) from random Voronoi states (2-6 regions, rho, p ~ U[0.1, 2], u, v ~ U[-1, 1]) with MUSCL2 + MOOD,
    SSP-RK3. Odd clouds: BGK-type discrete-velocity relaxation, 16 velocities on the unit ring, epsilon 1e-4, one
    macro moment advected with (1, 0.5), implicit source by IMEX ARS(2,2,2), from the Maxwellian of smooth random
    Fourier densities (the local relaxation initialisation of test/kinetic_source.jl:110-131). FP32 bulk. One context per system holds its whole batch (hcc_upload_batch: one cell list, one captured step
    graph per step), one dt per batch (its minimum CFL step)."""
    learned = sys.modules["hcc_gb300.learned"]
    rng = np.random.default_rng(2026)
    nc = args.ensemble_clouds
    target = np.exp(rng.uniform(np.log(4000.0), np.log(256000.0), nc))
    sides = np.maximum(8, np.rint(np.sqrt(target)).astype(int) - 1)
    h = 1.0 / 256
    t0 = time.time()
    ring = [(float(np.cos(2 * np.pi * q / 16)), float(np.sin(2 * np.pi * q / 16))) for q in range(16)]
    bgk = hcc.KineticRelaxation(ring, epsilon=1e-4, macro_velocity=(1.0, 0.5))
    groups = {"euler": [], "bgk": []}
    states = {"euler": [], "bgk": []}
    for k in range(nc):
        L = sides[k] * h
        cl = hcc.rectangular_cloud((0.0, 0.0), (L, L), h, 2.5 * h, jitter=0.25 * h, seed=1000 + k)
        xl = cl.pos / L
        if k % 2 == 0:
            groups["euler"].append(cl)
            states["euler"].append(learned.voronoi_state(xl, seed=k))
        else:
            r = np.random.default_rng(50000 + k)
            rho = np.ones(cl.n)
            for _ in range(3):
                kx, ky = r.integers(1, 4, 2)
                rho += 0.1 * r.uniform(0.5, 1.0) * np.sin(2 * np.pi * (kx * xl[:, 0] + ky * xl[:, 1]) + r.uniform(0, 6.3))
            groups["bgk"].append(cl)
            states["bgk"].append(bgk.maxwellian(rho))
    out = {"workload": f"ensemble_{nc}_clouds_2d", "clouds": nc, "setup": {}}
    totals = {}
    for name in ("euler", "bgk"):
        cl0 = groups[name][0]
        mood = hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h))
        bc = {t: hcc.BC_OUTFLOW for t in range(1, 5)}
        if name == "euler":
            cfg = hcc.make_config(hcc.Euler(2, 1.4), cl0, scheme=hcc.MUSCL(2, 2), mood=mood, tableau="RK3_SSP",
                                  bc_map=bc, precision="fp32")
            stages = 3
        else:
            cfg = hcc.make_config(bgk, cl0, scheme=hcc.MUSCL(2, 2), mood=mood, tableau="IMEX_ARS222",
                                  bc_map=bc, precision="fp32")
            stages = 3          # ARS(2,2,2): three stages (ButcherTableaus.jl:218-229)
        ctx = hcc.Context(cfg)
        ts = time.time()
        union = ctx.upload_batch(groups[name])
        ctx.build_neighbours()
        ctx.prepare_geometry()
        U = np.concatenate(states[name]).astype(np.float32)
        ctx.upload_state(U)
        dt = 0.4 * ctx.time_step()
        for _ in range(2):
            ctx.step(0.0, dt)
        ctx.upload_state(U)
        tune = ctx.autotune(dt, steps=2) if AUTOTUNE else None
        with ClockSampler(local) as clk:
            ms, launches = time_device_steps(hcc, ctx, dt, args.ensemble_steps, world)
        c = ctx.counters()
        n_int = int((union.is_boundary == 0).sum())
        totals[name] = (n_int * stages * args.ensemble_steps, ms)
        out[name] = {"clouds": len(groups[name]), "particles": union.n, "interior": n_int,
                     "ms_per_step": ms / args.ensemble_steps, "stages": stages, "dt": dt, "gpu_launches": launches,
                     "mood_iterations_last_step": c["mood_iterations"], "graph_steps": c["graph_steps"],
                     "setup_s": time.time() - ts, "clocks": clk.summary(), "tuning": tune}
        ctx.close()
    units = sum(u for u, _ in totals.values())
    ms_total = sum(m for _, m in totals.values())
    out["value"] = units * world / (ms_total / 1e3)
    out["unit"] = "point-updates/s per RK stage (both batches, interior particles)"
    out["generation_s"] = time.time() - t0
    return out


def run_profile_case(args):
    """Fixed workloads for kernel profilers (no timing, no JSON contract): `learned` / `plain` run
    `--profile-steps` host-driven steps of the bench workload with / without the shipped predictor; `predictor`
    runs the predictor's kernels on their own (1M random feature rows through the network, one 9728-row
    forward/backward pass) and then three host-driven steps with the predictor."""
    hcc = package()
    import torch
    torch.cuda.set_device(0)
    cloud, U0, h = make_workload(hcc, args.workload)
    pred = load_predictor(hcc)
    if args.profile == "predictor":
        rng = np.random.default_rng(0)
        X = np.abs(rng.normal(0.0, 0.5, (1 << 20, 24))).astype(np.float32)
        pred.predict_rows(X)
        n = 128 * 152 * 8 // 16
        pred.loss_grad(X[:n], (rng.random(n) < 0.4).astype(np.uint8))
    steps = 3 if args.profile == "predictor" else args.profile_steps
    ctx = hcc.Context(make_cfg(hcc, cloud, h, "fp32"))
    ctx.upload_cloud(cloud)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    ctx.upload_state(U0.astype(np.float32))
    if args.profile != "plain":
        ctx.set_predictor(pred, PREDICTOR_THRESHOLD)
    ctx.set_step_graphs(False)
    dt = 0.4 * ctx.time_step()
    for _ in range(steps):
        ctx.step(0.0, dt)
    ctx.synchronize()
    print(json.dumps({"profile": args.profile, "steps": steps, "counters": ctx.counters()}), flush=True)


def run_gpu(args):
    world, rank, local = dist_setup()
    hcc = package()
    if not hcc.LIB_PATH.exists():
        _load("hcc_gb300_build", PKG / "build.py").build()
    import torch
    torch.cuda.set_device(local)
    cloud, U0, h = make_workload(hcc, args.workload)
    D = cloud.pos.shape[1]
    n_int = cloud.n_interior
    results = {}
    acc_steps, acc_dt = 10, None
    predictor = None if args.no_learned else load_predictor(hcc)
    arms = ["fp32", "fp64"] if not args.fp32_only else ["fp32"]
    if predictor is not None:
        arms = ["fp32_learned"] + arms
    for arm in arms:
        prec = "fp64" if arm == "fp64" else "fp32"
        pr = predictor if arm == "fp32_learned" else None
        results[arm] = measure(hcc, cloud, U0, h, prec, args.steps, args.warmup, world, local,
                               acc_dt=acc_dt, acc_steps=acc_steps if acc_dt else 0, predictor=pr)
        if acc_dt is None:
            acc_dt = results[arm]["dt"]
            r = measure(hcc, cloud, U0, h, prec, 1, 0, world, local, e2e=False, acc_dt=acc_dt, acc_steps=acc_steps,
                        predictor=pr)
            results[arm]["rho"] = r["rho"]
    head = "fp32_learned" if predictor is not None else "fp32"
    r = results[head]
    units = n_int * STAGES * args.steps * world
    value = units / (r["ms"] / 1e3)
    cnt = r["counters"]
    K = cnt["total_neighbours"] / max(cloud.n, 1)
    M = D + 2
    flux_b, gather_b = algorithmic_bytes(K, D, M, D, D + 1, 4)
    peak, peak_kind = measured_peaks()
    kt = r["kt"]
    flux_ms = kt["flux_ms"] / max(kt["flux_launches"], 1)
    achieved = flux_b * n_int / (flux_ms / 1e3) / 1e9
    traffic = recorded_traffic().get("flux_f32_euler2d_bytes_per_point_stage") if D == 2 else None
    # the reconstruction pre-pass against the same peak: model bytes, and the DRAM bytes of its ncu capture
    gather_ms = kt["gather_ms"] / max(kt["gather_launches"], 1)
    g_traffic = recorded_traffic().get("gather_f32_euler2d_bytes_per_point_stage") if D == 2 else None
    g_model = gather_b * n_int / (gather_ms / 1e3) / 1e9
    gather_roof = {"kernel": f"k_gather<float,{D},{M},EULER,1>", "bound": "hbm", "unit": "GB/s", "peak": peak,
                   "achieved": g_model, "frac": g_model / peak,
                   "dram_achieved": (g_traffic * n_int / (gather_ms / 1e3) / 1e9) if g_traffic else None,
                   "dram_frac": (g_traffic * n_int / (gather_ms / 1e3) / 1e9 / peak) if g_traffic else None,
                   "note": "achieved: model bytes / live launch time; dram_achieved: ncu DRAM bytes per point-stage "
                           "(profiles/traffic.txt) x N_interior / live launch time"}
    line = {
        "metric": METRIC, "value": value, "unit": "point-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice)",
        "config": {"workload": args.workload, "description": WORKLOADS[args.workload][2],
                   "n_particles": cloud.n, "n_interior": n_int, "mean_neighbours": K, "stages_per_step": STAGES,
                   "precision": "FP32 bulk (FP64 MLS assembly/Cholesky)", "learned_mood": predictor is not None,
                   "predictor": ({"weights": "hypercloudcore.jl_gb300/predictor_euler2d.npz (train_predictor.py: "
                                  "200 seeded Voronoi runs at 250k nodes to t = 0.2)",
                                  "threshold": PREDICTOR_THRESHOLD} if predictor is not None else None),
                   "step_form": "one CUDA graph per step (MOOD fixed points as conditional WHILE nodes)",
                   "l2": "inputs larger than L2 (per-slot arrays ~0.5 GB)", "parallelism": f"replicas x{world}",
                   "dt": r["dt"], "launch_shapes": r["tuning"]},
        "gpu_launches": r["launches"],
        "e2e": {"value": units / r["e2e_s"], "unit": "point-updates/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"]},
        "roofline": {"bound": "hbm", "kernel": f"k_flux<float,{D},{M},EULER,1>", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": (traffic * n_int) if traffic else None,
                     "algorithmic_bytes_per_point_stage": {"flux": flux_b, "gather": gather_b},
                     "flux_ms_per_launch": flux_ms,
                     "gather_ms_per_launch": kt["gather_ms"] / max(kt["gather_launches"], 1),
                     "recompute_ms_total": kt["recompute_ms"], "recompute_launches": kt["recompute_launches"],
                     "predict_ms_per_step": kt["predict_ms"] / max(kt["steps"], 1),
                     "kernel_times": "CUDA events around each launch of a separate host-driven run of the same steps",
                     "gather": gather_roof},
        "clocks": r["clocks"],
        "mood": {"flagged_last_step": cnt["mood_flagged"], "iterations_last_step": cnt["mood_iterations"],
                 "predicted_last_step": cnt.get("predicted", 0)},
    }
    if head != "fp32":
        r0 = results["fp32"]
        line["fp32_plain"] = {"value": units / (r0["ms"] / 1e3), "ms_per_step": r0["ms"] / args.steps,
                              "e2e": units / r0["e2e_s"], "gpu_launches": r0["launches"],
                              "mood": {"flagged_last_step": r0["counters"]["mood_flagged"],
                                       "iterations_last_step": r0["counters"]["mood_iterations"]}}
    if "fp64" in results:
        r64 = results["fp64"]
        line["fp64_plain"] = {"value": units / (r64["ms"] / 1e3), "ms_per_step": r64["ms"] / args.steps,
                              "flux_ms_per_launch": r64["kt"]["flux_ms"] / max(r64["kt"]["flux_launches"], 1),
                              "gather_ms_per_launch": r64["kt"]["gather_ms"] / max(r64["kt"]["gather_launches"], 1),
                              "e2e": units / r64["e2e_s"], "clocks": r64["clocks"]}
        line["fp32_over_fp64"] = line["value"] / line["fp64_plain"]["value"]
        inner = cloud.is_boundary == 0
        line["l1_density_fp32_vs_fp64"] = {"value": rel_l1(results["fp32"]["rho"], r64["rho"], inner),
                                           "steps": acc_steps, "dt": acc_dt,
                                           "note": "relative L1 over interior particles, same dt"}
        if head != "fp32":
            line["l1_density_learned_vs_fp64"] = {"value": rel_l1(r["rho"], r64["rho"], inner), "steps": acc_steps,
                                                  "dt": acc_dt}
        if not args.no_reference_solution and D == 2:
            ref = fine_reference(hcc, cloud, h, acc_dt, acc_steps)
            acc = {"reference": "FP64 plain at h/2 (4x the particles), 2x the steps at dt/2, nearest fine particle",
                   "steps": acc_steps, "l1_fp64": rel_l1(r64["rho"], ref, inner),
                   "l1_fp32": rel_l1(results["fp32"]["rho"], ref, inner)}
            if head != "fp32":
                acc["l1_fp32_learned"] = rel_l1(r["rho"], ref, inner)
                acc["learned_over_fp64"] = acc["l1_fp32_learned"] / acc["l1_fp64"]
            acc["fp32_over_fp64"] = acc["l1_fp32"] / acc["l1_fp64"]
            line["accuracy_vs_finer_fp64"] = acc
    if not args.no_published:
        line["published_case"] = run_published_case(hcc, args.steps)
    if not args.no_3d and D == 2:
        line["euler3d_blast_8M"] = run_3d(hcc, args, world, local)
    if not args.no_ensemble and D == 2:
        line["ensemble"] = run_ensemble(hcc, args, world, local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(hcc, cloud, U0, h, args.cpu_steps)
    if rank == 0:
        print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------------------------- published case
# The reference's own benchmark (benchmark/step.jl, defaults): scalar advection with speeds (1, 0.5) on a uniform
# periodic 1000 x 1000 cloud, R = 2.5dx, MUSCL3 + VenkatakrishnanLimiter(:hard) + MOOD(EPD1, MOODu1(1e-6)), SSP-RK3,
# dt = 0.3 x get_time_step. Published ms/step on an RX 9070 XT / i5-13600K (8 cores): gpu_roadmap.md:215.
PUBLISHED_1M = {"f64_gpu_ms": 29.0, "f32_gpu_ms": 9.8, "f64_cpu8_ms": 387.0, "f32_cpu8_ms": 284.0,
                "hardware": "AMD RX 9070 XT (GPU), i5-13600K 8 cores (CPU)"}


def run_published_case(hcc, steps, n_side=1000):
    import torch
    h = 1.0 / n_side
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, periodic=True)
    U0 = np.exp(-((cloud.pos - 0.5) ** 2).sum(axis=1) / 0.02)[:, None].copy()
    out = {"workload": f"advection2d_muscl3_vk_mood_periodic_{n_side}x{n_side}", "n_particles": cloud.n,
           "published": PUBLISHED_1M}
    for prec in ("fp32", "fp64"):
        cfg = hcc.make_config(hcc.LinearAdvection(((1.0,), (0.5,))), cloud, scheme=hcc.MUSCL(3, 0, "vk_hard"),
                              mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-6)), precision=prec)
        ctx = hcc.Context(cfg)
        ctx.upload_cloud(cloud)
        ctx.build_neighbours()
        ctx.prepare_geometry()
        ctx.upload_state(U0.astype(np.float32) if prec == "fp32" else U0)
        dt = 0.3 * ctx.time_step()
        for _ in range(3):
            ctx.step(0.0, dt)
        stream = torch.cuda.ExternalStream(ctx.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ctx.synchronize()
        e0.record(stream)
        for _ in range(steps):
            ctx.step(0.0, dt)
        e1.record(stream)
        ctx.synchronize()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[f"{prec}_ms_per_step"] = ms
        out[f"{prec}_point_updates_per_s"] = 3 * cloud.n / (ms / 1e3)
        ctx.close()
    out["speedup_vs_published_gpu"] = {"f32": PUBLISHED_1M["f32_gpu_ms"] / out["fp32_ms_per_step"],
                                       "f64": PUBLISHED_1M["f64_gpu_ms"] / out["fp64_ms_per_step"]}
    return out


# --------------------------------------------------------------------------------------------- CPU (reference) arm
def cpu_baseline(hcc, cloud, U0, h, steps, warmup=1):
    """The oracle (C++ restatement of the reference CPU path, OpenMP on all host cores) on a bounded sample:
    `steps` steps of the same cloud after `warmup` warm-up steps."""
    orc = _load("hcc_oracle_py", ROOT / "oracle" / "oracle.py")
    abi = sys.modules["hcc_gb300._abi"]
    cores = os.cpu_count() or 1
    orc.load(abi)
    orc.OracleContext.set_threads(cores)
    o = orc.OracleContext(make_cfg(hcc, cloud, h, "fp64"), abi)
    o.upload_cloud(cloud)
    o.build_neighbours()
    o.prepare_geometry()
    o.upload_state(U0)
    dt = 0.4 * o.time_step()
    for _ in range(warmup):
        o.step(0.0, dt)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step(0.0, dt)
    el = time.perf_counter() - t0
    v = cloud.n_interior * STAGES * steps / el
    o.close()
    return {"value": v, "unit": "point-updates/s", "cores": cores, "kind": "port",
            "sample": f"{steps} SSP-RK3 step(s) of the full {cloud.n}-particle cloud after {warmup} warm-up "
                      f"step(s), FP64"}


def run_reference(args):
    world, rank, local = (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
                          int(os.environ.get("LOCAL_RANK", "0")))
    if rank != 0:
        return
    hcc = package()
    cloud, U0, h = make_workload(hcc, args.workload)
    # K timed and W warm-up steps of the whole cloud (about 0.6 s each on 16 Arm cores)
    steps, warmup = max(1, args.steps), max(0, args.warmup)
    base = cpu_baseline(hcc, cloud, U0, h, steps, warmup)
    line = {"metric": METRIC, "value": base["value"], "unit": "point-updates/s", "n_gpus": world, "steps": steps,
            "warmup": warmup, "ms_per_step": cloud.n_interior * STAGES / base["value"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered lattice)",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload][2],
                       "n_particles": cloud.n, "n_interior": cloud.n_interior},
            "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "point-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "Julia is not available on this box; the reference CPU path is its C++ restatement (oracle/)"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="euler2d_quadrant_1M", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp32-only", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="no troubled-point predictor (plain FP32 headline)")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched 512-cloud ensemble")
    ap.add_argument("--profile", choices=["learned", "plain", "predictor"], default=None,
                    help="run a fixed workload for a kernel profiler instead of the benchmark")
    ap.add_argument("--profile-steps", type=int, default=4)
    ap.add_argument("--ensemble-clouds", type=int, default=512)
    ap.add_argument("--ensemble-steps", type=int, default=5)
    ap.add_argument("--no-reference-solution", action="store_true", help="skip the h/2 FP64 reference run")
    ap.add_argument("--no-published", action="store_true")
    ap.add_argument("--no-3d", action="store_true")
    ap.add_argument("--host-driven", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes instead of hcc_autotune's")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    global HOST_DRIVEN, AUTOTUNE
    HOST_DRIVEN = args.host_driven
    AUTOTUNE = not args.no_autotune
    if args.profile:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

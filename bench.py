"""Throughput of the explicit right-hand-side path: point-updates/s per RK stage.

Workload (default, `euler3d_blast_8M`): 3-D compressible Euler, gamma 1.4, on [0,1]^3, jittered lattice h = 1/200
(±0.25h), 8.0M interior particles plus 0.85M ghosts, about 66 neighbours each within R = 2.5h; spherical blast
(rho = 1, p = 1 for r < 0.2 about the centre, else rho = 0.125, p = 0.1, zero velocity); transmissive (outflow)
boundaries; MUSCL order 2 with the MLS divergence fit of order 2; MOOD (EPD1, MOODu1 with delta = 1e-4 h^3);
Rusanov flux; SSP-RK3; dt = 0.4 x the CFL step at the initial state. Synthetic, seeded inputs (no dataset).

`value` is the FP32 bulk path with the learned troubled-point predictor attached (the headline; the plain FP32
path is `fp32_plain`), measured over --steps steps after --warmup warm-up steps with the state resident in HBM;
`e2e` is the same metric through the C ABI with host buffers (state uploaded from pinned memory and downloaded every
step); `fp64_plain` is the plain FP64 path on the same cloud over the same --steps/--warmup. `roofline` rates the
flux pass (and, under `roofline.gather`, the reconstruction pre-pass) against the measured HBM copy peak, with the
DRAM bytes per point-stage of the committed ncu capture (`profiles/traffic.txt`) as `traffic`. Every FP32 context is
tuned by `hcc_autotune` before its timed region (`--no-autotune`: default shapes). `euler2d_quadrant_1M`,
`published_case` and `ensemble` add the 2-D quadrant Riemann problem at 1.0M interior particles, the reference's own
benchmark case and the 512-cloud batched ensemble. `cpu_baseline` times the CPU oracle (the C++ restatement of the
reference's CPU path) on a bounded sample of the same workload; `--impl reference` runs only that CPU path.
`--study accuracy` runs the equal-L1 study at the configurations' end times instead (minutes; not part of the
default run).

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
TILE_STAGING = True     # --no-tile-staging: stream-fed FP32 full passes instead of the tile-staged ones
FORCE_TILES = False     # --tile-staging: tile-staged passes also where the library's default is stream-fed (2-D)


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
    "euler3d_blast_262k": (3, 1 / 64, "3-D Euler spherical blast, h=1/64 (262k interior), MUSCL2+MOOD, SSP-RK3"),
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


def make_cfg(hcc, cloud, h, precision, scheme=None):
    """MUSCL order 2 with the divergence fit of order 2 (or `scheme`), MOOD (EPD1, MOODu1(1e-4 h^D)), Rusanov,
    SSP-RK3, transmissive boundaries on every wall."""
    D = cloud.pos.shape[1]
    return hcc.make_config(hcc.Euler(D, 1.4), cloud, scheme=scheme if scheme is not None else hcc.MUSCL(2, 2),
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
def time_device_steps(hcc, ctx, dt, steps, world, dts=None):
    """K steps with the state resident in HBM, CUDA events on the context's stream, max over ranks (`dts`: a batch
    stepped with one dt per cloud)."""
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
        if dts is None:
            ctx.step(0.0, dt)
        else:
            ctx.step_batch(0.0, dts)
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


def _predictor_threshold():
    """One threshold for every workload, chosen on held-out training states, never on a test metric: the table of
    `train_predictor.py --holdout-eval` (held-out seeds, every row kept) -- the lowest threshold with precision
    >= 0.9 (a wrong pre-lowering costs accuracy, a missed one only a recompute). Returns (threshold, rule,
    qualified): when no threshold of the table qualifies, or the table is absent, the learned arm runs at 0.9 (the
    training run's choice) for comparison only and `qualified` is False, which keeps it out of the headline."""
    p = PKG / "predictor_euler2d_holdout.json"
    if p.exists():
        d = json.loads(p.read_text())
        if d.get("threshold"):
            return float(d["threshold"]), ("lowest held-out threshold with precision >= %g (held-out seeds, every row "
                                           "kept; predictor_euler2d_holdout.json)" % d["min_precision"]), True
        best = max(d["table"].items(), key=lambda kv: kv[1]["precision"])
        return 0.9, ("no held-out threshold reaches precision >= %g (held-out seeds, every row kept; best %.2f at "
                     "%s, recall %.2f): the training run's 0.9, for comparison only"
                     % (d["min_precision"], best[1]["precision"], best[0], best[1]["recall"])), False
    return 0.9, "the training run's threshold (no held-out table present), for comparison only", False


PREDICTOR_THRESHOLD, PREDICTOR_THRESHOLD_RULE, PREDICTOR_QUALIFIED = _predictor_threshold()


def measure(hcc, cloud, U0, h, prec, steps, warmup, world, local, *, e2e_steps=None, profile_steps=None,
            acc_dt=None, acc_steps=0, predictor=None, autotune=None):
    """One precision on one workload: `warmup` untimed steps, `steps` device-timed steps (the step graph, no
    profiling), `profile_steps` steps again with per-kernel CUDA events (host-driven) for the roofline, `e2e_steps`
    steps of the end-to-end C-ABI leg, and -- when asked -- `acc_steps` steps from the initial state with a fixed dt
    whose final density is returned for the L1 checks. With a predictor, every step pre-lowers the particles it
    predicts troubled (MOOD still judges every particle)."""
    f32 = prec == "fp32"
    e2e_steps = steps if e2e_steps is None else e2e_steps
    profile_steps = steps if profile_steps is None else profile_steps
    autotune = (AUTOTUNE and f32) if autotune is None else autotune
    ctx = hcc.Context(make_cfg(hcc, cloud, h, prec))
    if predictor is not None:
        ctx.set_predictor(predictor, PREDICTOR_THRESHOLD)
    if HOST_DRIVEN:
        ctx.set_step_graphs(False)
    t0 = time.perf_counter()
    ctx.upload_cloud(cloud)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    ctx.synchronize()
    setup_s = time.perf_counter() - t0
    if not TILE_STAGING or FORCE_TILES:
        ctx.set_tile_staging(TILE_STAGING and FORCE_TILES)
    U_in = U0.astype(np.float32) if f32 else U0
    ctx.upload_state(U_in)
    dt = 0.4 * ctx.time_step()
    t0 = time.perf_counter()
    for _ in range(5):
        ctx.time_step()
    cfl_ms = (time.perf_counter() - t0) / 5 * 1e3
    tune = ctx.autotune(dt, steps=3) if autotune and steps > 0 else None
    out = {"dt": dt, "tuning": tune, "setup_s": setup_s, "tile_staging": ctx.tile_staging(), "cfl_ms": cfl_ms}
    if steps > 0:
        ctx.upload_state(U_in)
        for _ in range(warmup):
            ctx.step(0.0, dt)
        with ClockSampler(local) as clk:
            ms, launches = time_device_steps(hcc, ctx, dt, steps, world)
        out.update({"ms": ms, "launches": launches, "clocks": clk.summary(), "counters": ctx.counters()})
    if profile_steps > 0:
        ctx.upload_state(U_in)
        ctx.set_profiling(True)
        ctx.kernel_times(reset=True)
        for _ in range(profile_steps):
            ctx.step(0.0, dt)
        ctx.synchronize()
        ctx.set_profiling(False)
        out["kt"] = ctx.kernel_times(reset=True)
    if e2e_steps > 0:
        out["e2e_s"], out["h2d"], out["d2h"] = time_e2e(hcc, ctx, U0, dt, e2e_steps, world, f32)
        out["e2e_steps"] = e2e_steps
    if acc_steps:
        ctx.upload_state(U_in)
        for _ in range(acc_steps):
            ctx.step(0.0, dt if acc_dt is None else acc_dt)
        out["rho"] = ctx.download_state(dtype=np.float64)[:, 0].copy()
        out["acc_counters"] = ctx.counters()
    ctx.close()
    return out


def rel_l1(a, b, sel):
    return float(np.abs(a[sel] - b[sel]).sum() / np.abs(b[sel]).sum())


def per_launch(kt, name):
    return kt[f"{name}_ms"] / max(kt[f"{name}_launches"], 1)


def roofline_of(workload, D, M, K, n_int, kt, peak, peak_kind, tiled=False):
    """The flux pass (dominant kernel) and the reconstruction pre-pass against the HBM copy peak: algorithmic bytes
    per point-stage x interior points / CUDA-event launch time; `traffic` = the ncu DRAM bytes per point-stage of
    profiles/traffic.txt for this workload, scaled to the launch. `tiled`: the tile-staged passes ran."""
    flux_b, gather_b = algorithmic_bytes(K, D, M, D, D + 1, 4)
    rec = recorded_traffic()
    flux_ms, gather_ms = per_launch(kt, "flux"), per_launch(kt, "gather")
    achieved = flux_b * n_int / (flux_ms / 1e3) / 1e9
    traffic = rec.get(f"flux_f32_{workload}_bytes_per_point_stage")
    g_traffic = rec.get(f"gather_f32_{workload}_bytes_per_point_stage")
    g_model = gather_b * n_int / (gather_ms / 1e3) / 1e9
    gname = f"k_gather_tile<{D},{M},EULER>" if tiled else f"k_gather<float,{D},{M},EULER,1>"
    fname = f"k_flux_tile<{D},{M},EULER>" if tiled else f"k_flux<float,{D},{M},EULER,1>"
    gather_roof = {"kernel": gname, "bound": "hbm", "unit": "GB/s", "peak": peak,
                   "achieved": g_model, "frac": g_model / peak,
                   "traffic": (g_traffic * n_int) if g_traffic else None,
                   "dram_achieved": (g_traffic * n_int / (gather_ms / 1e3) / 1e9) if g_traffic else None,
                   "dram_frac": (g_traffic * n_int / (gather_ms / 1e3) / 1e9 / peak) if g_traffic else None,
                   "ms_per_launch": gather_ms}
    return {"bound": "hbm", "kernel": fname, "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
            if peak_kind == "measured" else peak_kind,
            "traffic": (traffic * n_int) if traffic else None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per point-stage (profiles/traffic.txt)"
                              " x interior points",
            "algorithmic_bytes_per_point_stage": {"flux": flux_b, "gather": gather_b},
            "limiter": ("FP32 instruction issue, not HBM: 68 % issue-active, FMA pipe 47 %, DRAM traffic 1.1x the model "
                        "bytes (ncu, profiles/stage_f32_euler3d_blast_262k_tile.md)") if tiled else
                       ("issue / latency (ncu, profiles/stage_f32_euler2d_quadrant_1M.md)"),
            "flux_ms_per_launch": flux_ms, "gather_ms_per_launch": gather_ms,
            "recompute_ms_total": kt["recompute_ms"], "recompute_launches": kt["recompute_launches"],
            "predict_ms_per_step": kt["predict_ms"] / max(kt["steps"], 1),
            "kernel_times": "CUDA events on the context's stream around each launch of a separate host-driven run "
                            "of the same steps",
            "gather": gather_roof}


def fp64_roofline(D, M, K, n_int, kt, fp64_peak):
    """The FP64 flux pass against the FP64 pipe: FP64 operations per slot counted from the source (fp64_flops_per_slot)
    x slots / CUDA-event launch time."""
    if not kt or not kt.get("flux_launches"):
        return None
    flops = fp64_flops_per_slot(D, M)
    ms = per_launch(kt, "flux")
    achieved = flops * K * n_int / (ms / 1e3) / 1e12
    return {"bound": "fp64", "kernel": f"k_flux<double,{D},{M},EULER,1>", "flops_per_slot": flops,
            "achieved": achieved, "unit": "TFLOP/s", "peak": fp64_peak.get("tflops") if fp64_peak else None,
            "frac": (achieved / fp64_peak["tflops"]) if fp64_peak and fp64_peak.get("tflops") else None,
            "peak_source": fp64_peak.get("source") if fp64_peak else None, "flux_ms_per_launch": ms,
            "gather_ms_per_launch": per_launch(kt, "gather")}


def fp64_flops_per_slot(D, M):
    """FP64 operations (an FMA counts 2, a division or square root 1) of one slot of the FP64 MUSCL2 Euler flux pass
    (flux_one in hcc_stage_impl.cuh, compiled without contraction): two interface reconstructions (2 M D mul+add),
    two Euler flux/speed evaluations (each: 1 div, D mul + D-1 fma-pairs for |u|^2, 3 for p, 1 div + 1 sqrt + 2 mul
    for c, D(D+1) + 2D + D products for F, 2D for lambda), per axis the Rusanov flux (max, M jumps, M x 5) and the
    weighted accumulation (2 M D), the extrema (2 M)."""
    recon = 2 * (2 * M * D)
    euler = 2 * (1 + D + 2 * (D - 1) + 1 + 3 + 4 + D * (D + 1) + 2 * D + D + 2 * D)
    rusanov = D * (1 + M * 5)
    accum = 2 * M * D + M
    extrema = 2 * M
    return recon + euler + rusanov + accum + extrema


def run_ensemble(hcc, args, world, local):
    """Batched ensemble: `args.ensemble_clouds` independent 2-D clouds (default 512) with log-uniform node counts in
    [4k, 256k] (seeded), one spacing h = 1/256, jittered lattices with transmissive walls. Even clouds: Euler
    (gamma 1.4) from random Voronoi states (2-6 regions, rho, p ~ U[0.1, 2], u, v ~ U[-1, 1]) with MUSCL2 + MOOD,
    SSP-RK3. Odd clouds: BGK-type discrete-velocity relaxation, 16 velocities on the unit ring, epsilon 1e-4, one
    macro moment advected with (1, 0.5), implicit source by IMEX ARS(2,2,2), from the Maxwellian of smooth random
    Fourier densities (the local relaxation initialisation of test/kinetic_source.jl:110-131). FP32 bulk. One context per system holds its whole batch (hcc_upload_batch: one cell list, one captured step
    graph per step), one dt per cloud (each cloud's own CFL step, hcc_batch_step)."""
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
        dts = 0.4 * ctx.batch_time_steps()          # one dt per cloud (each cloud's own CFL step)
        for _ in range(2):
            ctx.step_batch(0.0, dts)
        ctx.upload_state(U)
        tune = ctx.autotune(dt, steps=2) if AUTOTUNE else None
        ctx.upload_state(U)
        with ClockSampler(local) as clk:
            ms, launches = time_device_steps(hcc, ctx, dt, args.ensemble_steps, world, dts=dts)
        c = ctx.counters()
        n_int = int((union.is_boundary == 0).sum())
        totals[name] = (n_int * stages * args.ensemble_steps, ms)
        out[name] = {"clouds": len(groups[name]), "particles": union.n, "interior": n_int,
                     "ms_per_step": ms / args.ensemble_steps, "stages": stages, "gpu_launches": launches,
                     "dt_per_cloud": {"min": float(dts.min()), "median": float(np.median(dts)), "max": float(dts.max())},
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
    prec = args.profile_precision
    scheme = hcc.WENO(2) if args.profile_scheme == "weno" else None
    ctx = hcc.Context(make_cfg(hcc, cloud, h, prec, scheme=scheme))
    ctx.upload_cloud(cloud)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    ctx.upload_state(U0.astype(np.float32) if prec == "fp32" else U0)
    if not TILE_STAGING or FORCE_TILES:
        ctx.set_tile_staging(TILE_STAGING and FORCE_TILES)
    if args.profile != "plain" and prec == "fp32":
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
    t_gen = time.perf_counter()
    cloud, U0, h = make_workload(hcc, args.workload)
    t_gen = time.perf_counter() - t_gen
    D = cloud.pos.shape[1]
    M = D + 2
    n_int = cloud.n_interior
    inner = cloud.is_boundary == 0
    K_steps, W = args.steps, args.warmup
    predictor = None if args.no_learned else load_predictor(hcc)
    fp64_steps = K_steps if args.fp64_steps is None else args.fp64_steps
    # the headline arm first; each arm also runs `acc` steps from the initial state at one shared dt (the first
    # arm's) for the density L1 distances between the arms
    acc, acc_dt = 5, None
    arms = (["fp32_learned"] if predictor is not None else []) + ["fp32"] + ([] if args.fp32_only else ["fp64"])
    res = {}
    for arm in arms:
        prec = "fp64" if arm == "fp64" else "fp32"
        kw = {}
        if prec == "fp64":          # ~1.4 s a step at 8M: no tuning (launch shapes are FP32 choices), short legs
            kw = {"profile_steps": min(fp64_steps, 2), "e2e_steps": min(fp64_steps, 2)}
        r = measure(hcc, cloud, U0, h, prec, fp64_steps if prec == "fp64" else K_steps, W if prec == "fp32" else
                    min(W, 3), world, local, acc_dt=acc_dt, acc_steps=acc,
                    predictor=predictor if arm == "fp32_learned" else None, **kw)
        if acc_dt is None:
            acc_dt = r["dt"]                 # the first arm's acc run used its own dt: the shared one
        res[arm] = r
    # the headline is the fastest FP32 arm at equal L1 with the FP64 path (the metric's condition): the arm with the
    # predictor when its threshold qualified on held-out data and the recorded study at the configured end time puts
    # its density error within 1.1x of FP64's at that threshold, else the plain FP32 arm (equal L1 at 1.00x)
    ratio, ratio_src = learned_l1_ratio(args.workload, PREDICTOR_THRESHOLD)
    head = "fp32_learned" if ("fp32_learned" in res and PREDICTOR_QUALIFIED and ratio is not None
                              and ratio <= 1.1) else "fp32"
    r = res[head]
    units = n_int * STAGES * K_steps * world
    value = units / (r["ms"] / 1e3)
    cnt = r["counters"]
    K = cnt["total_neighbours"] / max(cloud.n, 1)
    peak, peak_kind = measured_peaks()
    line = {
        "metric": METRIC, "value": value, "unit": "point-updates/s", "n_gpus": world, "steps": K_steps,
        "warmup": W, "ms_per_step": r["ms"] / K_steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice)",
        "config": {"workload": args.workload, "description": WORKLOADS[args.workload][2],
                   "n_particles": cloud.n, "n_interior": n_int, "mean_neighbours": K, "stages_per_step": STAGES,
                   "precision": "FP32 bulk (FP64 MLS assembly/Cholesky)", "learned_mood": head == "fp32_learned",
                   "headline_rule": "fastest FP32 arm whose density L1 at the configured end time is within 1.1x of "
                                    "the FP64 path's (the metric's equal-L1 condition)",
                   "predictor": ({"weights": "hypercloudcore.jl_gb300/predictor_euler2d.npz (train_predictor.py: "
                                  "200 seeded Voronoi runs at 250k nodes to t = 0.2)",
                                  "threshold": PREDICTOR_THRESHOLD,
                                  "threshold_rule": PREDICTOR_THRESHOLD_RULE}
                                 if head == "fp32_learned" else None),
                   "step_form": "one CUDA graph per step (MOOD fixed points as conditional WHILE nodes)",
                   "l2": "inputs larger than L2 (per-slot neighbour arrays of several GB)",
                   "parallelism": f"replicas x{world}", "dt": r["dt"], "launch_shapes": r["tuning"],
                   "setup_s": r["setup_s"], "cloud_generation_s": t_gen, "tile_staging": r["tile_staging"]},
        "gpu_launches": r["launches"],
        "e2e": {"value": n_int * STAGES * r["e2e_steps"] * world / r["e2e_s"], "unit": "point-updates/s",
                "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"], "steps": r["e2e_steps"]},
        "roofline": roofline_of(args.workload, D, M, K, n_int, r["kt"], peak, peak_kind,
                                tiled=bool(r["tile_staging"] and r["tile_staging"].get("active"))),
        "clocks": r["clocks"],
        "mood": {"flagged_last_step": cnt["mood_flagged"], "iterations_last_step": cnt["mood_iterations"],
                 "predicted_last_step": cnt.get("predicted", 0)},
        "cfl_ms_per_call": r["cfl_ms"],
    }
    other = "fp32" if head == "fp32_learned" else ("fp32_learned" if "fp32_learned" in res else None)
    if other:
        r0 = res[other]
        key = "fp32_plain" if other == "fp32" else "fp32_learned"
        line[key] = {"value": units / (r0["ms"] / 1e3), "ms_per_step": r0["ms"] / K_steps,
                     "e2e": n_int * STAGES * r0["e2e_steps"] * world / r0["e2e_s"],
                     "gpu_launches": r0["launches"], "clocks": r0["clocks"],
                     "flux_ms_per_launch": per_launch(r0["kt"], "flux"),
                     "gather_ms_per_launch": per_launch(r0["kt"], "gather"),
                     "mood": {"flagged_last_step": r0["counters"]["mood_flagged"],
                              "iterations_last_step": r0["counters"]["mood_iterations"],
                              "predicted_last_step": r0["counters"].get("predicted", 0)}}
        lv = res["fp32_learned"]["ms"] if "fp32_learned" in res else None
        if lv is not None:
            line["learned_over_plain"] = res["fp32"]["ms"] / lv
            line["learned_equal_l1"] = {"threshold": PREDICTOR_THRESHOLD, "threshold_rule": PREDICTOR_THRESHOLD_RULE,
                                        "threshold_qualified": PREDICTOR_QUALIFIED,
                                        "l1_over_fp64_at_end_time": ratio, "source": ratio_src,
                                        "meets_1_1x": ratio is not None and ratio <= 1.1,
                                        "headline": head == "fp32_learned"}
    if "fp64" in res:
        r64 = res["fp64"]
        u64 = n_int * STAGES * fp64_steps * world
        line["fp64_plain"] = {"value": u64 / (r64["ms"] / 1e3), "ms_per_step": r64["ms"] / fp64_steps,
                              "steps": fp64_steps, "warmup": min(W, 3),
                              "e2e": n_int * STAGES * r64["e2e_steps"] * world / r64["e2e_s"],
                              "clocks": r64["clocks"], "setup_s": r64["setup_s"],
                              "roofline": fp64_roofline(D, M, K, n_int, r64.get("kt"), fp64_peak(hcc))}
        line["fp32_over_fp64"] = line["value"] / line["fp64_plain"]["value"]
        for arm in arms:
            if arm != "fp64":
                line[f"l1_density_{arm}_vs_fp64"] = {"value": rel_l1(res[arm]["rho"], r64["rho"], inner),
                                                     "steps": acc, "dt": acc_dt,
                                                     "note": "relative L1 over interior particles, same dt"}
    rec = recorded_accuracy()
    if rec:
        line["accuracy_vs_finer_fp64"] = rec
    if not args.no_weno and D == 3:
        line["weno_variant"] = run_weno_variant(hcc, cloud, U0, h, K_steps, world, local)
    if not args.no_2d and D == 3:
        line["euler2d_quadrant_1M"] = run_secondary(hcc, args, world, local, "euler2d_quadrant_1M", predictor,
                                                    peak, peak_kind)
    if not args.no_published:
        line["published_case"] = run_published_case(hcc, K_steps)
    if not args.no_ensemble:
        line["ensemble"] = run_ensemble(hcc, args, world, local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(hcc, args.workload, args.cpu_steps)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_secondary(hcc, args, world, local, name, predictor, peak, peak_kind):
    """Another workload in the same line: FP32 (+ predictor) and FP64 step rates, the flux roofline."""
    cloud, U0, h = make_workload(hcc, name)
    D = cloud.pos.shape[1]
    n_int = cloud.n_interior
    K_steps = args.steps
    out = {"workload": name, "description": WORKLOADS[name][2], "n_particles": cloud.n, "n_interior": n_int}
    for arm in (["fp32_learned"] if predictor is not None else []) + ["fp32", "fp64"]:
        prec = "fp64" if arm == "fp64" else "fp32"
        r = measure(hcc, cloud, U0, h, prec, K_steps, args.warmup, world, local, e2e_steps=0,
                    profile_steps=min(K_steps, 3) if prec == "fp64" else K_steps,
                    predictor=predictor if arm == "fp32_learned" else None)
        units = n_int * STAGES * K_steps * world
        K = r["counters"]["total_neighbours"] / max(cloud.n, 1)
        out[arm] = {"value": units / (r["ms"] / 1e3), "ms_per_step": r["ms"] / K_steps, "clocks": r["clocks"],
                    "mood_iterations_last_step": r["counters"]["mood_iterations"]}
        if prec == "fp32":
            out[arm]["roofline"] = roofline_of(name, D, D + 2, K, n_int, r["kt"], peak, peak_kind,
                                               tiled=bool(r["tile_staging"] and r["tile_staging"].get("active")))
        else:
            out[arm]["roofline"] = fp64_roofline(D, D + 2, K, n_int, r.get("kt"), fp64_peak(hcc))
        out["mean_neighbours"] = K
    return out


def learned_l1_ratio(workload, thr):
    """The recorded density-L1 ratio (predictor arm over FP64 at the configured end time) of a workload at a
    threshold: the learned-only study (profiles/accuracy_learned.json), else the full study when it ran at that
    threshold; (None, why) when neither recorded it."""
    p = ROOT / "profiles" / "accuracy_learned.json"
    if p.exists():
        d = json.loads(p.read_text()).get(workload, {}).get("learned", {})
        if f"{thr:g}" in d:
            return d[f"{thr:g}"]["over_fp64"], "profiles/accuracy_learned.json"
    p = ROOT / "profiles" / "accuracy_equal_l1.json"
    if p.exists():
        d = json.loads(p.read_text())
        if abs(float(d.get("threshold", -1)) - thr) < 1e-12 and workload in d and "learned_over_fp64" in d[workload]:
            return d[workload]["learned_over_fp64"], "profiles/accuracy_equal_l1.json"
    return None, "no recorded study at this threshold"


def run_weno_variant(hcc, cloud, U0, h, steps, world, local):
    """The configuration's meshless-WENO variant of the same workload: component-wise WENO of order 2 for the Euler
    system (local Lax-Friedrichs splitting) with the same MOOD, SSP-RK3 and boundaries, FP32 and FP64 from the same
    state (the step graph, CUDA events; one step for FP64, whose fits run in FP64 at every stage)."""
    out = {"scheme": "meshless WENO order 2, component-wise (local Lax-Friedrichs splitting), MOOD EPD1/MOODu1",
           "note": "FP32: fit operators cached per stencil (FP64 assembly and Cholesky once per geometry), FP32 "
                   "gradients per stage; FP64: the oracle's order, fits assembled and factorised at every stage"}
    n_int = cloud.n_interior
    for prec, K, W in (("fp32", min(steps, 10), 2), ("fp64", 1, 0)):   # an FP64 step takes ~45 s at 8M
        ctx = hcc.Context(make_cfg(hcc, cloud, h, prec, scheme=hcc.WENO(2)))
        ctx.upload_cloud(cloud)
        ctx.build_neighbours()
        ctx.prepare_geometry()
        ctx.upload_state(U0.astype(np.float32) if prec == "fp32" else U0)
        dt = 0.4 * ctx.time_step()
        for _ in range(W):
            ctx.step(0.0, dt)
        with ClockSampler(local) as clk:
            ms, launches = time_device_steps(hcc, ctx, dt, K, world)
        out[prec] = {"ms_per_step": ms / K, "value": n_int * STAGES * K * world / (ms / 1e3), "steps": K,
                     "warmup": W, "gpu_launches": launches, "clocks": clk.summary(),
                     "mood_iterations_last_step": ctx.counters()["mood_iterations"]}
        ctx.close()
    out["fp32_over_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    return out


def recorded_accuracy():
    """The equal-L1 study's last recorded result (profiles/accuracy_equal_l1.json, written by --study accuracy)."""
    p = ROOT / "profiles" / "accuracy_equal_l1.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    d["source"] = "recorded by `python bench.py --study accuracy` (profiles/accuracy_equal_l1.json)"
    q = ROOT / "profiles" / "accuracy_learned.json"
    if q.exists():                       # the later sweep's plain FP32 arm (same references and end times)
        for name, r in json.loads(q.read_text()).items():
            if isinstance(r, dict) and "fp32_plain" in r and name in d:
                d[name]["fp32_over_fp64_recheck"] = r["fp32_plain"]["over_fp64"]
                d[name]["recheck_source"] = "profiles/accuracy_learned.json"
    return d


_FP64_PEAK = {}


def fp64_peak(hcc):
    """The FP64 FMA rate of this GPU, measured once per run (hcc_fp64_fma_rate)."""
    if "tflops" not in _FP64_PEAK:
        try:
            _FP64_PEAK["tflops"] = hcc.fp64_fma_rate()
            _FP64_PEAK["source"] = "measured: hcc_fp64_fma_rate (FP64 FMA chains on every SM, CUDA events)"
        except Exception as e:        # noqa: BLE001 - the roofline then has no peak
            _FP64_PEAK["tflops"] = None
            _FP64_PEAK["source"] = f"unavailable: {e}"
    return _FP64_PEAK


# --------------------------------------------------------------------------------------------- equal-L1 study
def radial_blast_reference(t_end, r_query, gamma=1.4, n=10000, r_max=0.9):
    """Density of the spherical blast (rho = 1, p = 1 for r < 0.2, else 0.125 / 0.1, at rest) at time t_end and radii
    r_query, from a fine 1-D solve in spherical symmetry (FP64): finite volumes on n cells of [0, r_max] with the
    geometric pressure source, minmod-limited linear reconstruction, Rusanov fluxes, SSP-RK3 at CFL 0.4, mirror
    condition at r = 0 and transmissive at r_max. Valid while the outer wave stays inside the unit cube's inscribed
    ball (t_end well below 0.15)."""
    dr = r_max / n
    rf = np.arange(n + 1) * dr
    rc = 0.5 * (rf[:-1] + rf[1:])
    A = rf ** 2
    V = (rf[1:] ** 3 - rf[:-1] ** 3) / 3.0
    dA = A[1:] - A[:-1]
    rho = np.where(rc < 0.2, 1.0, 0.125)
    pr = np.where(rc < 0.2, 1.0, 0.1)
    U = np.stack([rho, np.zeros(n), pr / (gamma - 1)])
    mirror = np.array([[1.0], [-1.0], [1.0]])

    def prim(U):
        r = U[0]
        u = U[1] / r
        return r, u, (gamma - 1) * (U[2] - 0.5 * r * u * u)

    def minmod(a, b):
        return np.where(a * b > 0, np.sign(a) * np.minimum(np.abs(a), np.abs(b)), 0.0)

    def flux(r, u, p):
        E = p / (gamma - 1) + 0.5 * r * u * u
        return np.stack([r, r * u, u * r * u + p, u * (E + p)]), np.stack([r * u, r * u * u + p, u * (E + p)])

    def rhs(U):
        r, u, p = prim(U)
        W = np.stack([r, u, p])
        Wg = np.concatenate([W[:, 1::-1] * mirror, W, np.repeat(W[:, -1:], 2, axis=1)], axis=1)
        d = np.diff(Wg, axis=1)
        s = minmod(d[:, :-1], d[:, 1:])                  # slopes of columns 1 .. n+2
        WL = Wg[:, 1:n + 2] + 0.5 * s[:, 0:n + 1]        # faces 0 .. n
        WR = Wg[:, 2:n + 3] - 0.5 * s[:, 1:n + 2]
        cL, FL = flux(WL[0], WL[1], WL[2])
        cR, FR = flux(WR[0], WR[1], WR[2])
        UL = np.stack([WL[0], WL[0] * WL[1], WL[2] / (gamma - 1) + 0.5 * WL[0] * WL[1] ** 2])
        UR = np.stack([WR[0], WR[0] * WR[1], WR[2] / (gamma - 1) + 0.5 * WR[0] * WR[1] ** 2])
        sm = np.maximum(np.abs(WL[1]) + np.sqrt(gamma * WL[2] / WL[0]), np.abs(WR[1]) + np.sqrt(gamma * WR[2] / WR[0]))
        F = 0.5 * (FL + FR) - 0.5 * sm * (UR - UL)
        AF = A * F
        out = -(AF[:, 1:] - AF[:, :-1]) / V
        out[1] += p * dA / V
        return out

    t = 0.0
    while t < t_end:
        r, u, p = prim(U)
        dt = min(0.4 * dr / np.max(np.abs(u) + np.sqrt(gamma * p / r)), t_end - t)
        U1 = U + dt * rhs(U)
        U2 = 0.75 * U + 0.25 * (U1 + dt * rhs(U1))
        U = U / 3.0 + 2.0 / 3.0 * (U2 + dt * rhs(U2))
        t += dt
    return np.interp(r_query, rc, U[0])


def run_cfl_steps(hcc, cloud, U0, h, prec, dts=None, steps=None, t_end=None, predictor=None, scheme=None):
    """Steps from the initial state: with `dts`, exactly those step sizes; otherwise dt = 0.4 x the CFL step of the
    current state until `steps` steps or time `t_end`. Returns (density, the dt sequence, MOOD flags summed over the
    steps, seconds)."""
    ctx = hcc.Context(make_cfg(hcc, cloud, h, prec, scheme=scheme))
    if predictor is not None:
        ctx.set_predictor(predictor, PREDICTOR_THRESHOLD)
    ctx.upload_cloud(cloud)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    ctx.upload_state(U0.astype(np.float32) if prec == "fp32" else U0)
    seq, t, flagged = [], 0.0, 0
    t0 = time.perf_counter()
    while True:
        if dts is not None:
            if len(seq) == len(dts):
                break
            dt = dts[len(seq)]
        else:
            if (steps is not None and len(seq) == steps) or (t_end is not None and t >= t_end * (1 - 1e-14)):
                break
            dt = 0.4 * ctx.time_step()
            if t_end is not None:
                dt = min(dt, t_end - t)
        ctx.step(t, dt)
        seq.append(dt)
        t += dt
        flagged += ctx.counters()["mood_flagged"]
    ctx.synchronize()
    el = time.perf_counter() - t0
    rho = ctx.download_state(dtype=np.float64)[:, 0].copy()
    ctx.close()
    return rho, seq, flagged, el


def run_accuracy_study(args):
    """Density L1 errors of FP64 plain, FP32 bulk and FP32 + predictor at the configurations' end times:
    the 3-D blast at 8.0M interior particles after 200 steps (dt = 0.4 x the FP64 path's CFL step each step, the
    same sequence replayed by the FP32 arms) against the fine 1-D radial solve at the same time; the 2-D quadrant
    problem at 1.0M interior particles at t = 0.25 against the FP64 path at h/2 (nearest fine particle)."""
    from scipy.spatial import cKDTree
    hcc = package()
    import torch
    torch.cuda.set_device(0)
    predictor = load_predictor(hcc)
    if args.study_learned_only:
        return run_learned_study(args, hcc, predictor, cKDTree)
    out = {"threshold": PREDICTOR_THRESHOLD}
    for name in args.study_workloads.split(","):
        cloud, U0, h = make_workload(hcc, name)
        D = cloud.pos.shape[1]
        inner = cloud.is_boundary == 0
        rec = {"workload": name}
        rho64, dts, f64, s64 = run_cfl_steps(hcc, cloud, U0, h, "fp64",
                                             steps=200 if D == 3 else None, t_end=None if D == 3 else 0.25)
        t_end = float(np.sum(dts))
        rec.update({"steps": len(dts), "t_end": t_end, "dt_first": dts[0], "dt_last": dts[-1]})
        if D == 3:
            r = np.sqrt(((cloud.pos - 0.5) ** 2).sum(axis=1))
            ref = radial_blast_reference(t_end, r)
            rec["reference"] = "1-D spherical FP64 solve (10,000 cells on [0, 0.9], Rusanov + minmod, SSP-RK3)"
        else:
            fine = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h / 2, 2.5 * h / 2, jitter=0.25 * h / 2, seed=42)
            Uf = quadrant_state(fine)
            rf, fdts, _, sf = run_cfl_steps(hcc, fine, Uf, h / 2, "fp64", t_end=t_end)
            _, idx = cKDTree(fine.pos).query(cloud.pos)
            ref = rf[idx]
            rec["reference"] = (f"FP64 plain at h/2 ({fine.n} particles), its own CFL steps ({len(fdts)}) to the same "
                                f"time, nearest fine particle")
            rec["reference_seconds"] = sf
        rec["l1_fp64"] = rel_l1(rho64, ref, inner)
        rec["fp64_seconds"] = s64
        rec["fp64_flagged_total"] = f64
        rho32, _, f32, s32 = run_cfl_steps(hcc, cloud, U0, h, "fp32", dts=dts)
        rec.update({"l1_fp32": rel_l1(rho32, ref, inner), "fp32_seconds": s32, "fp32_flagged_total": f32})
        rec["fp32_over_fp64"] = rec["l1_fp32"] / rec["l1_fp64"]
        if predictor is not None:
            rhol, _, fl, sl = run_cfl_steps(hcc, cloud, U0, h, "fp32", dts=dts, predictor=predictor)
            rec.update({"l1_fp32_learned": rel_l1(rhol, ref, inner), "fp32_learned_seconds": sl,
                        "fp32_learned_flagged_total": fl})
            rec["learned_over_fp64"] = rec["l1_fp32_learned"] / rec["l1_fp64"]
        out[name] = rec
        print(json.dumps({name: rec}), flush=True)
    print(json.dumps({"accuracy_study": out}), flush=True)
    if args.study_out:
        Path(args.study_out).write_text(json.dumps(out, indent=1) + "\n")


def run_weno_study(args):
    """Density L1 errors of the configuration's two schemes (MUSCL2 + MOOD, meshless WENO of order 2 + MOOD) in FP64
    and FP32 on the 3-D blast at the size where the FP64 WENO path, whose fits run in FP64 at every stage, is
    affordable (262k interior), at the recorded study's end time, against the 1-D radial FP64 solve."""
    hcc = package()
    import torch
    torch.cuda.set_device(0)
    rec = json.loads((ROOT / "profiles" / "accuracy_equal_l1.json").read_text())
    t_end = rec["euler3d_blast_8M"]["t_end"]
    name = "euler3d_blast_262k"
    cloud, U0, h = make_workload(hcc, name)
    inner = cloud.is_boundary == 0
    ref = radial_blast_reference(t_end, np.sqrt(((cloud.pos - 0.5) ** 2).sum(axis=1)))
    out = {"workload": name, "n_interior": int(cloud.n_interior), "t_end": t_end,
           "reference": "1-D spherical FP64 solve (radial_blast_reference)"}
    for label, scheme in (("muscl", hcc.MUSCL(2, 2)), ("weno", hcc.WENO(2))):
        for prec in ("fp64", "fp32"):
            rho, dts, flagged, sec = run_cfl_steps(hcc, cloud, U0, h, prec, t_end=t_end, scheme=scheme)
            out[f"{label}_{prec}"] = {"l1": rel_l1(rho, ref, inner), "steps": len(dts), "seconds": sec,
                                      "flagged_total": flagged}
            print(json.dumps({f"{label}_{prec}": out[f"{label}_{prec}"]}), flush=True)
        out[f"{label}_fp32_over_fp64"] = out[f"{label}_fp32"]["l1"] / out[f"{label}_fp64"]["l1"]
    print(json.dumps({"weno_study": out}), flush=True)
    if args.study_out:
        Path(args.study_out).write_text(json.dumps(out, indent=1) + "\n")


def run_learned_study(args, hcc, predictor, cKDTree):
    """The FP32 + predictor arm of the equal-L1 study again, for the thresholds of --study-thresholds (default: the
    held-out one), against the references of the recorded study (profiles/accuracy_equal_l1.json: its end times and
    FP64 errors; the references recomputed -- the radial solve, or the FP64 run at h/2, which is deterministic). Each
    run takes its own CFL steps (0.4) to the recorded end time."""
    global PREDICTOR_THRESHOLD
    rec = json.loads((ROOT / "profiles" / "accuracy_equal_l1.json").read_text())
    thresholds = [(x if x == "plain" else float(x)) for x in args.study_thresholds.split(",")] \
        if args.study_thresholds else [PREDICTOR_THRESHOLD]
    keep = PREDICTOR_THRESHOLD
    out = {"held_out_threshold": keep, "rule": PREDICTOR_THRESHOLD_RULE}
    for name in args.study_workloads.split(","):
        r0 = rec[name]
        cloud, U0, h = make_workload(hcc, name)
        D = cloud.pos.shape[1]
        inner = cloud.is_boundary == 0
        t_end = r0["t_end"]
        if D == 3:
            ref = radial_blast_reference(t_end, np.sqrt(((cloud.pos - 0.5) ** 2).sum(axis=1)))
        else:
            fine = hcc.rectangular_cloud((0.0,) * D, (1.0,) * D, h / 2, 2.5 * h / 2, jitter=0.25 * h / 2, seed=42)
            rf, _, _, _ = run_cfl_steps(hcc, fine, quadrant_state(fine), h / 2, "fp64", t_end=t_end)
            ref = rf[cKDTree(fine.pos).query(cloud.pos)[1]]
        res = {"t_end": t_end, "l1_fp64": r0["l1_fp64"], "learned": {}}
        for thr in thresholds:
            if thr == "plain":                  # the FP32 arm without the predictor, for comparison
                rho, dts, flagged, sec = run_cfl_steps(hcc, cloud, U0, h, "fp32", t_end=t_end)
                l1 = rel_l1(rho, ref, inner)
                res["fp32_plain"] = {"l1": l1, "over_fp64": l1 / r0["l1_fp64"], "steps": len(dts),
                                     "flagged_total": flagged, "seconds": sec}
                continue
            PREDICTOR_THRESHOLD = thr
            rho, dts, flagged, sec = run_cfl_steps(hcc, cloud, U0, h, "fp32", t_end=t_end, predictor=predictor)
            l1 = rel_l1(rho, ref, inner)
            res["learned"][f"{thr:g}"] = {"l1": l1, "over_fp64": l1 / r0["l1_fp64"], "steps": len(dts),
                                         "flagged_total": flagged, "seconds": sec}
        PREDICTOR_THRESHOLD = keep
        out[name] = res
        print(json.dumps({name: res}), flush=True)
    print(json.dumps({"learned_study": out}), flush=True)
    if args.study_out:
        Path(args.study_out).write_text(json.dumps(out, indent=1) + "\n")


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
def reference_sample(hcc, workload):
    """The bounded sample of a workload that the CPU path is timed on. 2-D: the whole cloud. The 3-D blast at 8.0M:
    the sub-box [0.25, 0.75]^3 at the same spacing and support radius (1.03M interior particles, the same ~66
    neighbours each, the same physics and scheme), which contains the whole initial blast sphere; the metric is per
    point-update, so the sample measures the same per-point cost at a size the CPU finishes in seconds per step."""
    D, h, _ = WORKLOADS[workload]
    if D == 2:
        cloud, U0, h = make_workload(hcc, workload)
        return cloud, U0, h, f"the full {cloud.n}-particle cloud"
    lo, hi = 0.25, 0.75
    cloud = hcc.rectangular_cloud((lo,) * D, (hi,) * D, h, 2.5 * h, jitter=0.25 * h, seed=42)
    return cloud, blast_state(cloud), h, (f"the sub-box [{lo}, {hi}]^3 of the workload at the same spacing "
                                          f"({cloud.n} particles, {cloud.n_interior} interior)")


def cpu_baseline(hcc, workload, steps, warmup=1):
    """The oracle (C++ restatement of the reference CPU path, OpenMP on all host cores, FP64) on a bounded sample of
    the workload: `steps` steps after `warmup` warm-up steps."""
    orc = _load("hcc_oracle_py", ROOT / "oracle" / "oracle.py")
    abi = sys.modules["hcc_gb300._abi"]
    cores = os.cpu_count() or 1
    orc.load(abi)
    orc.OracleContext.set_threads(cores)
    cloud, U0, h, what = reference_sample(hcc, workload)
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
            "sample": f"{steps} SSP-RK3 step(s) after {warmup} warm-up step(s) of {what}, FP64"}


def run_reference(args):
    world, rank, local = (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
                          int(os.environ.get("LOCAL_RANK", "0")))
    if rank != 0:
        return
    hcc = package()
    D, h, desc = WORKLOADS[args.workload]
    # K timed and W warm-up steps of the bounded sample (about 1-3 s a step on 16 Arm cores)
    steps, warmup = max(1, args.steps), max(0, args.warmup)
    base = cpu_baseline(hcc, args.workload, steps, warmup)
    line = {"metric": METRIC, "value": base["value"], "unit": "point-updates/s", "n_gpus": world, "steps": steps,
            "warmup": warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered lattice)",
            "config": {"workload": args.workload, "description": desc},
            "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "point-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "Julia is not available on this box; the reference CPU path is its C++ restatement (oracle/), "
                    "timed on a bounded sample of the workload (cpu_baseline.sample)"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="euler3d_blast_8M", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp32-only", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="no troubled-point predictor (plain FP32 headline)")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched 512-cloud ensemble")
    ap.add_argument("--profile", choices=["learned", "plain", "predictor"], default=None,
                    help="run a fixed workload for a kernel profiler instead of the benchmark")
    ap.add_argument("--profile-steps", type=int, default=4)
    ap.add_argument("--profile-precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--ensemble-clouds", type=int, default=512)
    ap.add_argument("--ensemble-steps", type=int, default=5)
    ap.add_argument("--no-reference-solution", action="store_true", help="skip the h/2 FP64 reference run")
    ap.add_argument("--no-published", action="store_true")
    ap.add_argument("--no-2d", action="store_true", help="skip the 2-D quadrant workload of a 3-D run")
    ap.add_argument("--no-weno", action="store_true", help="skip the meshless-WENO variant of a 3-D run")
    ap.add_argument("--fp64-steps", type=int, default=None, help="timed FP64 steps (default: --steps)")
    ap.add_argument("--study", choices=["accuracy", "weno"], default=None,
                    help="run the equal-L1 study at the configurations' end times (accuracy), or the MUSCL / WENO "
                         "comparison on the 262k blast (weno), instead of the benchmark")
    ap.add_argument("--study-workloads", default="euler3d_blast_8M,euler2d_quadrant_1M")
    ap.add_argument("--study-out", default=None, help="also write the study's JSON here")
    ap.add_argument("--study-learned-only", action="store_true",
                    help="only the FP32 + predictor arm, against the recorded study's references and end times")
    ap.add_argument("--study-thresholds", default=None,
                    help="comma-separated predictor thresholds (learned-only); 'plain' adds the FP32 arm without it")
    ap.add_argument("--host-driven", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes instead of hcc_autotune's")
    ap.add_argument("--profile-scheme", choices=["muscl", "weno"], default="muscl",
                    help="scheme of the profile runs (--profile plain)")
    ap.add_argument("--no-tile-staging", action="store_true", help="stream-fed FP32 full passes (A/B)")
    ap.add_argument("--tile-staging", action="store_true",
                    help="tile-staged FP32 passes also where the default is stream-fed (2-D; A/B)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    global HOST_DRIVEN, AUTOTUNE, TILE_STAGING, FORCE_TILES
    HOST_DRIVEN = args.host_driven
    AUTOTUNE = not args.no_autotune
    TILE_STAGING = not args.no_tile_staging
    FORCE_TILES = args.tile_staging
    if args.study == "accuracy":
        run_accuracy_study(args)
    elif args.study == "weno":
        run_weno_study(args)
    elif args.profile:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

"""Throughput of the GB300 terrain tile producer (elevation + normal tiles/s).

Workload (one step): a frame of 4096 independent tile requests, levels uniform in
1..12, 25% of them 197-wide and the rest 101-wide; every request has its own
materialised fBm parent tile (zf, zm planes), an iid N(0, (2000 * 0.5^l)^2)
residual tile and per-level noise 300 * 0.55^l m with the DEM noise table.
Each step produces the elevation (zf, zc, zm) and normal (nx, ny) tiles of all
requests.  The inputs of one step (about 1.8 GB) exceed the 129 MB L2, so no
flush is needed between steps.

  value  device-resident throughput: inputs already in HBM, job arrays already
         on the device, CUDA events around K steps on the launch stream.
  e2e    the same frame through the C ABI with host buffers: host->device copy
         of parents and residuals from pinned memory, the batch call (which
         also uploads its job array), device->host copy of all output tiles.

--impl reference times the reference's CPU path for this hot path (the C
restatement of CPUElevationProducer::doCreateTile plus the shader's noise, zc,
zm and normal arithmetic) on all host cores over the whole frame per step,
from inputs drawn with the same seeds; it loads the oracle only.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "proland-4.0_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "elev+normal tiles/s (101² and 197²), plain vs learned; max err vs FP64"
UNIT = "tiles/s"
ROOT_QUAD = 100000.0          # meters: terrainNode size 50000 -> root quad 2 * size
BYTES_PER_TILE = {101: 260960, 197: 1000544}   # algorithmic bytes (parent window, residual, elevation, normals)
FALLBACK_HBM_GBS = 6800.0
E2E_CHUNK = {101: 512, 197: 128}   # tiles per chunk of the host-buffer pipeline (swept: 64-512 / 16-128)
TRAFFIC_PROFILE = os.path.join(ROOT, "profiles", "frame_kernel_traffic.txt")


def traffic_per_tile():
    """DRAM bytes (read + write) per tile of each width, as measured by the ncu capture
    summarised in profiles/frame_kernel_traffic.txt (its `per_tile` line), or None."""
    try:
        with open(TRAFFIC_PROFILE) as f:
            for line in f:
                if line.startswith("per_tile"):
                    return {int(k[1:]): float(v) for k, v in (t.split("=") for t in line.split()[1:])}
    except (OSError, ValueError):
        pass
    return None


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ------------------------------------------------------------------ workload
def synthetic_inputs():
    """The numpy generator of the synthetic inputs (proland_gb300/workloads.py), loaded
    from its file: both arms draw the same seeded frame from it, and the reference arm
    does not import the package (nor, through it, the CUDA library)."""
    import importlib.util
    name = "tp_synthetic_inputs"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, os.path.join(PKG, "proland_gb300", "workloads.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        sys.modules[name] = mod
    return sys.modules[name]


class FrameClass:
    """All requests of one tile width, laid out in slots: outputs [0, n), parents [n, 2n).

    `select(face, level, tx, ty) -> (rotation, layer)` is the noise-layer choice of
    ElevationProducer.cpp:345-376: the library's for the GPU arm, the oracle's for the
    reference arm (the two are tested identical)."""

    def __init__(self, W, levels, tx, ty, seed, select, n_unique_parents=48):
        wl = synthetic_inputs()
        self.W, self.n = W, len(levels)
        self.levels, self.tx, self.ty = levels, tx, ty
        uz, um = wl.fbm_parent_tiles(min(n_unique_parents, self.n), W, seed)
        pick = np.arange(self.n) % uz.shape[0]
        self.parent_zf = uz[pick]
        self.parent_zm = um[pick]
        self.residual = wl.residual_tiles(levels, W, seed + 1)
        sel = [select(1, int(l), int(x), int(y)) for l, x, y in zip(levels, tx, ty)]
        self.noise_rot = np.array([r for r, _ in sel], np.int32)
        self.noise_layer = np.array([k for _, k in sel], np.int32)
        self.noise_amp = np.array([wl.noise_amplitude(int(l)) for l in levels], np.float32)
        self.tile_meters = np.array([ROOT_QUAD / (1 << int(l)) for l in levels], np.float32)
        self.jobs = None

    def make_jobs(self, tp):
        """The library's job records (tp_tile_job) of this class."""
        self.jobs = [tp.make_job(int(self.levels[k]), int(self.tx[k]), int(self.ty[k]), out_slot=k,
                                 parent_slot=self.n + k, residual_slot=k, normal_slot=k,
                                 noise_rot=int(self.noise_rot[k]), noise_layer=int(self.noise_layer[k]),
                                 noise_amp=float(self.noise_amp[k]), tile_meters=float(self.tile_meters[k]))
                     for k in range(self.n)]

    def allocate(self, tp):
        self.elev = tp.TileStorage(self.W, 3, 2 * self.n)
        self.res = tp.TileStorage(self.W, 1, self.n)
        self.nrm = tp.TileStorage(self.W - 4, 2, self.n)

    def upload_inputs(self, tp, stream=None):
        self.elev.upload(self.n, tp.ZF, self.h_parent_zf, stream)
        self.elev.upload(self.n, tp.ZM, self.h_parent_zm, stream)
        self.res.upload(0, 0, self.h_residual, stream)

    def run_host(self, tp, pipe, params, stream):
        """The whole frame of this width from host tiles to host tiles; parent zm is
        derived on the device from parent zf (max(zf, 0)), as the parent's own
        production wrote it."""
        pipe.run(params, self.jobs, self.h_parent_zf, None, self.h_residual, self.h_zf, self.h_zc, self.h_zm,
                 self.h_nx, self.h_ny, stream)

    def download_outputs(self, tp, stream=None):
        for c, buf in ((tp.ZF, self.h_zf), (tp.ZC, self.h_zc), (tp.ZM, self.h_zm)):
            self.elev.download(0, self.n, c, buf, stream)
        self.nrm.download(0, self.n, tp.NX, self.h_nx, stream)
        self.nrm.download(0, self.n, tp.NY, self.h_ny, stream)

    def pin(self, torch):
        W, n = self.W, self.n

        def pinned(shape):
            return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()
        self.h_parent_zf = pinned((n, W, W)); self.h_parent_zf[:] = self.parent_zf
        self.h_parent_zm = pinned((n, W, W)); self.h_parent_zm[:] = self.parent_zm
        self.h_residual = pinned((n, W, W)); self.h_residual[:] = self.residual
        self.h_zf, self.h_zc, self.h_zm = (pinned((n, W, W)) for _ in range(3))
        self.h_nx, self.h_ny = (pinned((n, W - 4, W - 4)) for _ in range(2))
        self.h2d_bytes = 2 * n * W * W * 4 + n * C.sizeof(self.jobs[0])   # parent zf, residual, jobs
        self.d2h_bytes = n * (3 * W * W + 2 * (W - 4) ** 2) * 4


def make_frame(nreq, seed, select):
    levels, tx, ty, wide = synthetic_inputs().frame_requests(nreq, seed)
    classes = []
    for W, sel in ((101, ~wide), (197, wide)):
        idx = np.nonzero(sel)[0]
        if len(idx):
            classes.append(FrameClass(W, levels[idx], tx[idx], ty[idx], seed + W, select))
    return classes


def frame_config(classes, world):
    """The `config` object both arms print for the frame workload."""
    alg = sum(fc.n * BYTES_PER_TILE[fc.W] for fc in classes)
    return {"workload": workload_name(classes), "form": "plain",
            "l2": "inputs larger than L2 (%.2f GB per step)" % (alg / 1e9),
            "parallelism": "replicas" if world > 1 else "single GPU"}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.proc = None
        self.path = None
        self.dev = device_index

    def start(self):
        try:
            import tempfile
            self.path = os.path.join(tempfile.gettempdir(), "bench_clocks_%d.csv" % os.getpid())
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the timed region starts once the sampler is running; its samples so far are
        # left out of the record
        t0 = time.time()
        self.skip = 0
        while time.time() - t0 < 5.0 and self.proc.poll() is None:
            self.f.flush()
            with open(self.path) as r:
                n = sum(1 for _ in r)
            if n > 0:
                self.skip = n
                break
            time.sleep(0.02)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        return clock_record(list(open(self.path))[self.skip:])


def clock_record(lines):
    """The `clocks` object of a run from nvidia-smi's CSV samples (ClockSampler.QUERY,
    noheader, nounits): median SM clock, the maximum, the throttle reasons seen active
    in any sample, the sample count; None without a readable sample."""
    sm, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in lines:
        parts = [p.strip() for p in line.split(",")]
        if len(parts) < 9:
            continue
        try:
            clk, top = float(parts[1]), float(parts[2])
        except ValueError:
            continue
        sm.append(clk)
        mx = top
        for nm, v in zip(names, parts[5:9]):
            if v.lower() == "active":
                reasons.add(nm)
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU path
def cpu_jobs(classes, outs_keepalive):
    """The oracle's job records (or_job) of every request of the frame, with host
    output tiles; the same inputs, noise choice and amplitudes as the device frame."""
    import oracle
    jobs = []
    fp = oracle._f32p
    for fc in classes:
        W, m = fc.W, fc.n
        table = oracle.dem_noise(W)
        zf = np.empty((m, W, W), np.float32); zc = np.empty_like(zf); zm = np.empty_like(zf)
        nx = np.empty((m, W - 4, W - 4), np.float32); ny = np.empty_like(nx)
        outs_keepalive += [table, zf, zc, zm, nx, ny]
        for k in range(m):
            b = oracle.Job()
            b.W, b.level, b.tx, b.ty = W, int(fc.levels[k]), int(fc.tx[k]), int(fc.ty[k])
            b.parent_zf = fc.parent_zf[k].ctypes.data_as(fp)
            b.parent_zm = fc.parent_zm[k].ctypes.data_as(fp)
            b.parent_pitch = W
            b.residual = fc.residual[k].ctypes.data_as(fp)
            b.res_pitch, b.rx, b.ry, b.rscale = W, 0, 0, 1.0
            b.noise = table[int(fc.noise_layer[k])].ctypes.data_as(fp)
            b.noise_rot, b.noise_amp = int(fc.noise_rot[k]), float(fc.noise_amp[k])
            b.tile_meters = float(fc.tile_meters[k])
            b.out_zf, b.out_zc, b.out_zm = (a[k].ctypes.data_as(fp) for a in (zf, zc, zm))
            b.out_pitch = W
            b.out_nx, b.out_ny = nx[k].ctypes.data_as(fp), ny[k].ctypes.data_as(fp)
            b.nrm_pitch = W - 4
            jobs.append(b)
    return jobs


def tuned_matches(jobs, sample=4):
    """The tuned build of the CPU path gives the same tiles as the oracle's own build."""
    import oracle
    pick = [jobs[0], next(j for j in jobs if j.W == 197)][:sample]

    def outputs(job):
        n, m = job.W * job.W, (job.W - 4) ** 2
        return ([np.ctypeslib.as_array(getattr(job, f), shape=(n,)).copy() for f in ("out_zf", "out_zc", "out_zm")]
                + [np.ctypeslib.as_array(getattr(job, f), shape=(m,)).copy() for f in ("out_nx", "out_ny")])
    oracle.run_jobs(pick, 1)
    want = [outputs(j) for j in pick]
    oracle.run_jobs(pick, 1, tuned=True)
    got = [outputs(j) for j in pick]
    return all(np.array_equal(a, b) for wa, ga in zip(want, got) for a, b in zip(wa, ga))


CPU_BUILD = "gcc -O3 -ffp-contract=off on this host (no machine-specific flags)"


def time_cpu(classes, min_seconds=4.0):
    """Tiles/s of the CPU path on all host threads: whole frames, repeated for about
    `min_seconds` (the GPU arm's `cpu_baseline`)."""
    import oracle
    from oracle import build as obuild
    obuild.build()
    threads = os.cpu_count() or 1
    keep = []
    jobs = cpu_jobs(classes, keep)
    same = tuned_matches(jobs)
    oracle.run_jobs(jobs[:4 * threads], threads, tuned=True)          # warm-up
    t0 = time.perf_counter()
    reps = 0
    while True:
        oracle.run_jobs(jobs, threads, tuned=True)
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    out = {"value": reps * len(jobs) / el, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": "the whole frame (%d tiles: %d x 101, %d x 197), %d repetitions, %.1f s" % (
               len(jobs), sum(1 for j in jobs if j.W == 101), sum(1 for j in jobs if j.W == 197), reps, el),
           "build": CPU_BUILD, "same_results_as_oracle": same}
    # one thread, the frame's 3:1 mix
    one = [j for j in jobs if j.W == 101][:12] + [j for j in jobs if j.W == 197][:4]
    t0 = time.perf_counter()
    reps = 0
    while time.perf_counter() - t0 < min_seconds / 2:
        oracle.run_jobs(one, 1, tuned=True)
        reps += 1
    out["single_thread"] = {"value": reps * len(one) / (time.perf_counter() - t0), "unit": UNIT, "cores": 1}
    out["residual_decode"] = residual_decode_rate()
    return out


def residual_decode_rate(min_seconds=1.0):
    """Host decode of residual tiles from the reference's DEM.dat pyramid (deflate
    TIFF strips, int16 x scale), the work ResidualProducer does per tile: the
    oracle's zlib-based decoder and the library's own inflate, tiles/s on one thread."""
    import oracle
    import proland_gb300 as tp
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "dem_terrain4_mini.dat")
    if not os.path.exists(path):
        return None
    d = oracle.DatFile.open(path)
    tiles = [(l, x, y) for l in range(0, d.max_level + 1) for x in range(1 << l) for y in range(1 << l)
             if (l >= d.min_level or (x == 0 and y == 0)) and d.tile_id(l, x, y) < d.ntiles
             and len(d.strip(l, x, y)) > 0]
    def rate(fn):
        t0 = time.perf_counter()
        k = 0
        while time.perf_counter() - t0 < min_seconds:
            for t in tiles:
                fn(*t)
                k += 1
        return k / (time.perf_counter() - t0)
    lib = tp.DatPyramid(path)
    res = {"oracle_zlib_tiles_per_s": rate(d.tile_int16), "library_inflate_tiles_per_s": rate(lib.tile_int16),
           "tiles": len(tiles), "tile_width": d.tile_size + 5, "file": "tests/golden/dem_terrain4_mini.dat"}
    lib.close()
    return res


def workload_name(classes):
    """The frame workload as both arms name it in their config."""
    return ("frame: %d independent requests per GPU, levels 1-12, %d x 101 + %d x 197 tiles, "
            "materialised fBm parents, residual sigma 2000*0.5^l, noise 300*0.55^l"
            % (sum(fc.n for fc in classes), sum(fc.n for fc in classes if fc.W == 101),
               sum(fc.n for fc in classes if fc.W == 197)))


def run_reference(args):
    """The reference's CPU path for this hot path (the oracle's restatement of
    CPUElevationProducer::doCreateTile with the shader's noise, zc, zm and normal
    arithmetic) over the whole frame per step, on all host threads.  Builds the frame
    from numpy and the oracle only: nothing of the GPU library is loaded."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    import oracle
    from oracle import build as obuild
    obuild.build()
    classes = make_frame(args.requests, args.seed, oracle.noise_select)
    threads = os.cpu_count() or 1
    keep = []
    jobs = cpu_jobs(classes, keep)
    same = tuned_matches(jobs)
    for _ in range(max(args.warmup, 1)):
        oracle.run_jobs(jobs, threads, tuned=True)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.run_jobs(jobs, threads, tuned=True)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = args.steps * len(jobs) / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": frame_config(classes, world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "the whole frame (%d tiles) per step" % len(jobs),
                             "build": CPU_BUILD, "same_results_as_oracle": same},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ------------------------------------------------------------------ GPU path
def check_host_outputs(classes, sample=16):
    """The host-buffer run's outputs against the device run's slots (same jobs and
    inputs): True when the sampled tiles are bit-identical in all five planes."""
    import proland_gb300 as tp
    for fc in classes:
        m = min(sample, fc.n)
        dev = [fc.elev.download(0, m, c) for c in (tp.ZF, tp.ZC, tp.ZM)] + \
              [fc.nrm.download(0, m, c) for c in (tp.NX, tp.NY)]
        host = (fc.h_zf, fc.h_zc, fc.h_zm, fc.h_nx, fc.h_ny)
        for d, h in zip(dev, host):
            if not np.array_equal(d, h[:m]):
                return False
    return True


def fp64_errors(tp, classes):
    """Max error of a few produced tiles against the FP64 evaluation of the same
    definition (and of the normals computed from FP64 elevations)."""
    import oracle
    out = {"zf_abs": 0.0, "zf_rel": 0.0, "normal_abs": 0.0, "tiles": 0,
           # reporting only: how far the GL path's LINEAR fetches at +0.25-texel offsets
           # would move the normals from the texel-exact finite differences computed here
           "normal_abs_vs_gl_linear_sampling": 0.0}
    for fc in classes:
        table = oracle.dem_noise(fc.W)
        for k in range(min(4, fc.n)):
            j = fc.jobs[k]
            zf = fc.elev.download(k, 1, tp.ZF)[0]
            nx = fc.nrm.download(k, 1, tp.NX)[0]
            d_zf, d_zc, d_zm = oracle.elevation_tile(
                fc.W, j.level, j.tx, j.ty, fc.parent_zf[k], fc.parent_zm[k], fc.residual[k],
                noise=table[j.noise_layer], noise_rot=j.noise_rot, noise_amp=j.noise_amp, f64=True)
            dnx, _ = oracle.normals_flat_f64(fc.W, d_zm, j.tile_meters)
            e = np.abs(zf.astype(np.float64) - d_zf)
            out["zf_abs"] = max(out["zf_abs"], float(e.max()))
            out["zf_rel"] = max(out["zf_rel"], float((e / np.maximum(np.abs(d_zf), 1.0)).max()))
            out["normal_abs"] = max(out["normal_abs"], float(np.abs(nx - dnx).max()))
            zm = fc.elev.download(k, 1, tp.ZM)[0]
            lnx, _ = oracle.normals_flat_gl_linear(fc.W, zm, j.tile_meters)
            out["normal_abs_vs_gl_linear_sampling"] = max(out["normal_abs_vs_gl_linear_sampling"],
                                                          float(np.abs(nx - lnx).max()))
            out["tiles"] += 1
    return out


# forward FLOPs of the learned net per W x W tile: 2 x samples x 9 taps x sum(cin x cout)
# over the used channels (4 -> 32, 3 x 32 -> 32, 32 -> 1), and as executed on the tensor
# cores (padded channels 16 -> 32, 32 -> 16; 8 x 16 pixel blocks covering the tile)
def learned_flops(W):
    used = 2 * W * W * 9 * (4 * 32 + 3 * 32 * 32 + 32 * 1)
    rows = ((W + 7) // 8) * ((W + 15) // 16) * 128
    executed = 2 * rows * 9 * (16 * 32 + 3 * 32 * 32 + 32 * 16)
    return used, executed


# HBM bytes of one W x W tile's forward pass as the kernels move them: the input channels
# made from the upsampled tile (fp32 read, 16 bf16 channels written), then per layer the
# bf16 activations of (W + 2)^2 pixels read (zero border included) and W^2 written, the
# last layer's fp32 channel, and the residual scaled out (fp32 read and write)
def learned_bytes(W):
    """HBM bytes per W x W tile of an inference pass: the tile means, the first layer
    (its input channels made from the fp32 upsampled tile), three hidden layers, the
    last layer and the output scaling."""
    px, pxb = W * W, (W + 2) * (W + 2)
    b = px * 4                                # tile means
    b += px * 4 + px * 32 * 2                 # layer 0 (upsampled tile in, 32 channels out)
    b += 3 * (pxb * 32 * 2 + px * 32 * 2)     # layers 1-3 (32 -> 32)
    b += pxb * 32 * 2 + px * 4                # layer 4 (32 -> 1 used)
    b += 2 * px * 4                           # scale
    return b


ORTHO_W = 196
ORTHO_BYTES_PER_TILE = 4 * ((ORTHO_W // 2 + 2) ** 2 + 2 * ORTHO_W * ORTHO_W)   # parent window, residual, output


def ortho_section(tp, torch, stream, sh, args):
    """Ortho (colour) tiles: a frame of 4096 independent 196-wide RGBA8 requests,
    levels 1-12, each with its own parent tile (48 distinct random parents cycled)
    and a stored residual (bytes around 128), HSV noise as terrain3 configures it
    (rnoise 60,150,20, cnoise 70,80,100, amplitude 255 at every level).  One
    persistent launch per step; CUDA events on the launch stream."""
    import oracle
    W, n = ORTHO_W, 4096
    rng = np.random.default_rng(args.seed + 3)
    levels = rng.integers(1, 13, n)
    tx = np.array([rng.integers(0, 1 << int(l)) for l in levels])
    ty = np.array([rng.integers(0, 1 << int(l)) for l in levels])
    pool = rng.integers(0, 256, (48, W, W, 4), dtype=np.uint8)
    rpool = np.clip(rng.normal(128.0, 20.0, (64, W, W, 4)), 0, 255).astype(np.uint8)
    orth = tp.TileStorage(W, 1, 2 * n)
    res = tp.TileStorage(W, 1, n)
    idx = np.arange(n)
    orth.upload(n, 0, tp.rgba_to_texels(pool[idx % 48]), sh)
    res.upload(0, 0, tp.rgba_to_texels(rpool[idx % 64]), sh)
    params = tp.make_ortho_params(root_color=(60 / 255, 150 / 255, 20 / 255, 1.0),
                                  noise_color=(70 / 255, 80 / 255, 100 / 255, 1.0), scale=2.0,
                                  hsv=not args.ortho_rgb)
    jobs = []
    for k in range(n):
        l = int(levels[k])
        rot, layer = tp.noise_select(1, l, int(tx[k]), int(ty[k]))
        jobs.append(tp.make_ortho_job(l, int(tx[k]), int(ty[k]), out_slot=k, parent_slot=n + k, residual_slot=k,
                                      noise_rot=rot, noise_layer=layer, noise_amp=255.0))
    arr = (tp.OrthoJob * n)(*jobs)
    dev_jobs = torch.empty(C.sizeof(arr), dtype=torch.uint8, device="cuda")
    dev_jobs.copy_(torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8))
    torch.cuda.synchronize()
    jp = C.c_void_p(dev_jobs.data_ptr())
    for _ in range(max(args.warmup, 3)):
        tp.ortho_batch_device(orth, res, params, jp, n, sh)
    steps = max(args.steps // 4, 10)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        tp.ortho_batch_device(orth, res, params, jp, n, sh)
    e1.record(stream)
    torch.cuda.synchronize()
    tp.stream_check(sh)
    ms = e0.elapsed_time(e1) / steps
    gbs = n * ORTHO_BYTES_PER_TILE / (ms / 1000.0) / 1e9
    peak, src = hbm_peak()
    # parity on sampled tiles against the oracle, and the oracle's single-thread rate
    table = oracle.ortho_noise(W)
    ok = True
    t0 = time.perf_counter()
    sample = [0, 1, n // 2, n - 1]
    for k in sample:
        j = jobs[k]
        want = oracle.ortho_tile(W, j.level, j.tx, j.ty, pool[k % 48], rpool[k % 64], table[j.noise_layer],
                                 j.noise_rot, j.noise_amp, root_color=list(params.root_color),
                                 noise_color=list(params.noise_color), scale=params.scale,
                                 hsv=bool(params.hsv))
        got = tp.texels_to_rgba(orth.download(k, 1, 0)[0])
        ok = ok and bool(np.array_equal(got, want))
    cpu_rate = len(sample) / (time.perf_counter() - t0)
    out = {"workload": "%d independent 196x196 RGBA8 ortho requests, levels 1-12, stored residuals, %s noise"
                       % (n, "HSV" if params.hsv else "RGB"),
           "tiles_per_s": n / (ms / 1000.0), "ms_per_step": ms, "steps": steps,
           "algorithmic_bytes_per_tile": ORTHO_BYTES_PER_TILE,
           "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                        "peak_source": src, "kernel": "ortho_kernel (one persistent launch)"},
           "identical_to_oracle_on_sample": ok,
           "cpu_single_thread_oracle_tiles_per_s": cpu_rate}
    orth.close()
    res.close()
    return out


def water_meshes(layers, rng, W, size=1000.0):
    """One tile of the water elevation layer (layers.water_layer): a lake of 9 points
    with a 6-point island (filled under the odd winding rule, both boundaries drawn),
    a crossing curve under NOTEQUAL and a 3-point river with caps under LESS."""
    def ring(cx, cy, r, n):
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        rad = r * rng.uniform(0.6, 1.0, n)
        return np.column_stack([cx + rad * np.cos(ang), cy + rad * np.sin(ang)])
    outer = ring(size * rng.uniform(0.3, 0.7), size * rng.uniform(0.3, 0.7), size * 0.3, 9)
    island = ring(outer[:, 0].mean(), outer[:, 1].mean(), size * 0.06, 6)
    curves = [([(-100.0, size * rng.uniform(0, 1)), (size + 100.0, size * rng.uniform(0, 1))],
               rng.uniform(0, 50, 2), float(rng.uniform(10, 60)))]
    river = ([(size * rng.uniform(-0.1, 1.1), -50.0), (size * rng.uniform(0.2, 0.8), size * rng.uniform(0.3, 0.7)),
              (size * rng.uniform(-0.1, 1.1), size + 50.0)], rng.uniform(-20, 80, 3), float(rng.uniform(8, 40)),
             True, True)
    ms = layers.water_layer((0.0, 0.0), size, W, areas=[[outer, island]],
                            boundaries=[(np.vstack([outer, outer[:1]]), 1), (np.vstack([island, island[:1]]), 0)],
                            curves=curves, rivers=[river])
    return [(v, ix, mode, i == 0, prog, state, fd) for i, (v, ix, mode, prog, state, fd) in enumerate(ms)]


def layer_pass_case(tp, torch, stream, sh, oracle, W, zf, zm, tiles, what):
    """One layer workload: parity of a sample against the oracle, then passes timed
    with CUDA events on the stream, meshes resident on the device and uploaded from
    pinned host memory."""
    n = len(tiles)
    elev = tp.TileStorage(W, 3, n)
    pick = np.arange(n) % len(zf)
    elev.upload(0, tp.ZF, zf[pick], sh)
    batch = tp.LayerBatch(tiles)
    ntri = 0
    for _, ms in tiles:
        for m in ms:
            cnt = len(m[1]) if m[1] is not None else len(m[0])
            ntri += cnt // 3 if m[2] == tp.TRIANGLES else max(cnt - 2, 0)
    # parity on a sample: one pass over fresh zm planes
    elev.upload(0, tp.ZM, zm[pick], sh)
    batch.run(elev, 0, sh)
    tp.stream_check(sh)
    ok = True
    t0 = time.perf_counter()
    sample = [0, 1, n // 2, n - 1]
    for k in sample:
        want = oracle.layer_tile(W, zf[pick[k]], zm[pick[k]], tiles[k][1], 0)
        ok = ok and bool(np.array_equal(elev.download(k, 1, tp.ZM, stream=sh)[0], want))
    cpu_rate = len(sample) / (time.perf_counter() - t0)
    batch.pin(torch).to_device(torch)

    def timed(fn, steps=10):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        tp.stream_check(sh)
        return e0.elapsed_time(e1) / steps
    ms_dev = timed(lambda: batch.run_device(elev, 0, sh))
    ms_host = timed(lambda: batch.run(elev, 0, sh))
    out = {"workload": "layer pass over %d produced %dx%d tiles, %s (%d triangles)" % (n, W, W, what, ntri),
           "tiles_per_s": n / (ms_dev / 1000.0), "triangles_per_s": ntri / (ms_dev / 1000.0),
           "ms_per_pass": ms_dev, "pass": "meshes resident on the device (tp_elevation_layers_device)",
           "host_meshes": {"ms_per_pass": ms_host, "tiles_per_s": n / (ms_host / 1000.0),
                           "mesh_bytes_uploaded_per_pass": batch.n_vertices * 16 + batch.n_indices * 4,
                           "pass": "meshes in pinned host memory, uploaded by each pass (tp_elevation_layers)"},
           "steps": 10, "texel_bytes_per_tile": 12 * W * W,
           "identical_to_oracle_on_sample": ok,
           "cpu_single_thread_oracle_tiles_per_s": cpu_rate}
    elev.close()
    return out


def layers_section(tp, torch, stream, sh, args):
    """Elevation layer passes (tp_elevation_layers) over 4096 produced 101-wide tiles,
    blended into zm (graph1 blend): the road layer, two roads per tile (3-point
    polylines, widths 5-40 m, on 1000 m tiles: strips of ~290 triangles, built by
    layers.road_strip); and the water layer (layers.water_layer: lake fill and
    boundaries under ALWAYS, a curve under NOTEQUAL, a river with caps under LESS;
    256 distinct tiles, repeated).  A pass uploads its meshes from host memory, then
    runs one CTA per tile; CUDA events on the stream around whole passes."""
    import oracle
    from proland_gb300 import layers
    W, n = 101, 4096
    rng = np.random.default_rng(args.seed + 5)
    zf = (rng.standard_normal((64, W, W)) * 200.0).astype(np.float32)
    zm = np.maximum(zf, np.float32(0.0))
    tiles = []
    for k in range(n):
        ms = []
        for r in range(2):
            a, b = rng.uniform(-200, 1200, 2), rng.uniform(-200, 1200, 2)
            mid = (a + b) / 2 + rng.uniform(-150, 150, 2)
            v = layers.road_strip([a, mid, b], rng.uniform(0, 300, 3), float(rng.uniform(5, 40)), (0.0, 0.0),
                                  1000.0, W)
            ms.append((v, None, tp.TRIANGLE_STRIP, r == 0))
        tiles.append((k, ms))
    out = layer_pass_case(tp, torch, stream, sh, oracle, W, zf, zm, tiles, "2 road strips each")
    distinct = [water_meshes(layers, rng, W) for _ in range(256)]
    out["water"] = layer_pass_case(tp, torch, stream, sh, oracle, W, zf, zm,
                                   [(k, distinct[k % 256]) for k in range(n)],
                                   "the water layer's passes (lake, island, curve, capped river)")
    return out


def quadtree_case(levels, W, seed_root=1):
    """Configuration 0's inputs: the tiles of a levels 0..`levels` quadtree (parents
    first), the root's residual an 8-octave fBm tile, level l's residuals
    N(0, (2000 * 0.5^l)^2) with seed 2 + l."""
    wl = synthetic_inputs()
    tiles = [(l, x, y) for l in range(levels + 1) for y in range(1 << l) for x in range(1 << l)]
    resid = np.empty((len(tiles), W, W), np.float32)
    resid[0] = wl.value_noise_fbm((W, W), octaves=8, seed=seed_root)
    k = 1
    for l in range(1, levels + 1):
        m = 4 ** l
        resid[k:k + m] = wl.residual_tiles([l] * m, W, seed=2 + l)
        k += m
    return tiles, resid


def quadtree_bytes(tiles, W):
    """Algorithmic bytes of producing `tiles` (the root has no parent window)."""
    return sum(BYTES_PER_TILE[W] - (2 * ((W - 5) // 2 + 5) ** 2 * 4 if l == 0 else 0) for l, _, _ in tiles)


def quadtree_section(tp, torch, stream, sh, args):
    """Configuration 0 as a timed frame: the whole levels 0-5 quadtree (1365 tiles of
    101^2, fBm root, residuals, noise off, normals for every tile) in ONE persistent
    launch whose jobs wait in the kernel for their parent's completion counter
    (parents before children), autotuned and replayed from a CUDA graph; beside it
    the same tiles as one launch per level (six launches in stream order, no
    in-kernel waits).  CUDA events on the launch stream around K whole quadtrees."""
    W, L, D = 101, 5, 50000.0
    tiles, resid = quadtree_case(L, W)
    n = len(tiles)
    index = {t: k for k, t in enumerate(tiles)}
    elev, res, nrm = tp.TileStorage(W, 3, n), tp.TileStorage(W, 1, n), tp.TileStorage(W - 4, 2, n)
    res.upload(0, 0, resid, sh)
    jobs = []
    for k, (l, x, y) in enumerate(tiles):
        pj = index[(l - 1, x // 2, y // 2)] if l > 0 else -1
        jobs.append(tp.make_job(l, x, y, out_slot=k, parent_slot=pj, residual_slot=k, normal_slot=k,
                                tile_meters=D / (1 << l), parent_job=pj))
    params = tp.make_params()
    steps = max(args.steps // 4, 20)
    alg = quadtree_bytes(tiles, W)
    peak, src = hbm_peak()

    def timed(run):
        with torch.cuda.stream(stream):
            for _ in range(5):
                run()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            run()
        e1.record(stream)
        torch.cuda.synchronize()
        tp.stream_check(sh)
        return e0.elapsed_time(e1) / steps

    one = tp.Frame()
    one.add(elev, res, nrm, params, jobs)
    one.autotune(sh, repeats=5)
    ms_one = timed(lambda: one.graph_launch(sh))
    shape = one.config(0)
    zf_one = elev.download(0, n, tp.ZF)
    waves = []
    first = 0
    for l in range(L + 1):
        m = 4 ** l
        f = tp.Frame()
        f.add(elev, res, nrm, params, [tp.make_job(j.level, j.tx, j.ty, out_slot=j.out_slot, parent_slot=j.parent_slot,
                                                   residual_slot=j.residual_slot, normal_slot=j.normal_slot,
                                                   tile_meters=j.tile_meters) for j in jobs[first:first + m]])
        f.autotune(sh, repeats=3)
        waves.append(f)
        first += m

    def run_waves():
        for f in waves:
            f.graph_launch(sh)
    ms_waves = timed(run_waves)
    same = bool(np.array_equal(elev.download(0, n, tp.ZF), zf_one))
    for f in waves:
        f.close()
    one.close()
    best = min(ms_one, ms_waves)
    gbs = alg / (best / 1000.0) / 1e9
    out = {"workload": "levels 0-%d quadtree, %d tiles of %dx%d, fBm root, residuals, noise off, normals" % (L, n, W, W),
           "tiles": n, "algorithmic_bytes": alg, "steps": steps,
           "one_launch": {"ms": ms_one, "tiles_per_s": n / (ms_one / 1000.0),
                          "achieved_gbs": alg / (ms_one / 1000.0) / 1e9,
                          "frac": alg / (ms_one / 1000.0) / 1e9 / peak, "shape": shape,
                          "form": "one persistent launch, parents before children, in-kernel waits on the "
                                  "parent's completion counter, CUDA graph"},
           "level_waves": {"ms": ms_waves, "tiles_per_s": n / (ms_waves / 1000.0),
                           "achieved_gbs": alg / (ms_waves / 1000.0) / 1e9,
                           "frac": alg / (ms_waves / 1000.0) / 1e9 / peak,
                           "form": "one launch per level (6), each a CUDA graph, in stream order"},
           "same_tiles": same,
           "tiles_per_s": n / (best / 1000.0),
           "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                        "peak_source": src}}
    elev.close(); res.close(); nrm.close()
    return out


def streaming_section(tp, torch, stream, sh, args):
    """Configuration 2 as timed frames: the seeded camera path of 600 frames from 10 km
    down to 50 m over a level 0-14 quadtree (root 50 km), 8192-slot caches, through the
    native TileSampler over the elevation and normal producers (tp_sampler_update:
    release the vanished quads' tiles, acquire the new ones, one scheduler run:
    synthetic residuals made on the device, one
    persistent elevation launch with the flat normals fused, parents first).  The
    frames' quadtree requests are generated before the timed run (TerrainQuad's split
    rule, timed apart); each frame is timed on the host around the update and a
    stream synchronisation, its device work by CUDA events on the stream."""
    from proland_gb300 import streaming as S
    W, slots, frames = 101, 8192, 600
    cams = S.camera_path(frames)
    t0 = time.perf_counter()
    reqs = [np.ascontiguousarray(np.asarray(S.quadtree_requests(c), np.int32)) for c in cams]
    req_ms = 1000.0 * (time.perf_counter() - t0) / frames
    amps = [300.0 * 0.55 ** l for l in range(S.MAX_LEVEL + 1)]

    def chain(n_slots, seed):
        rs, es, ns = tp.TileStorage(W, 1, n_slots), tp.TileStorage(W, 3, n_slots), tp.TileStorage(W - 4, 2, n_slots)
        rc, ec, nc = tp.TileCache(rs, "residual"), tp.TileCache(es, "elevation"), tp.TileCache(ns, "normal")
        r = tp.ResidualProducer(rc, synthetic=(2000.0, 0.5, seed))
        e = tp.ElevationProducer(ec, r, noise_amp=amps, params=tp.make_params(), face=0)
        n = tp.NormalProducer(nc, e)
        for p in (e, n):
            p.set_root_quad_size(S.ROOT_SIZE)
        return [rs, es, ns, rc, ec, nc, r, e, n], tp.TileSampler(e, n)

    L = tp.lib()
    n_new = C.c_int()

    def update(smp, a):
        rc = L.tp_sampler_update(smp.handle, a.ctypes.data_as(C.POINTER(C.c_int32)), a.shape[0], sh, C.byref(n_new))
        tp.check(rc)
        return n_new.value

    # warm-up: a few frames of the path on a separate chain
    objs, smp = chain(slots, args.seed + 11)
    for f in range(0, 40, 4):
        update(smp, reqs[f])
    stream.synchronize()
    smp.close()
    objs, smp = chain(slots, args.seed + 12)
    tp.trace_host_times(reset=True)
    old_flags = tp.trace_set(2)
    host_ms, dev_ms, news = [], [], []
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(frames)]
    torch.cuda.synchronize()
    t_all = time.perf_counter()
    for f in range(frames):
        t0 = time.perf_counter()
        evs[f][0].record(stream)
        news.append(update(smp, reqs[f]))
        evs[f][1].record(stream)
        stream.synchronize()
        host_ms.append(1000.0 * (time.perf_counter() - t0))
    total_ms = 1000.0 * (time.perf_counter() - t_all)
    tp.trace_set(old_flags)
    phases = {k: {"ms_per_frame": 1000.0 * v[0] / frames, "calls": v[1]}
              for k, v in tp.trace_host_times(reset=True).items() if v[1]}
    tp.stream_check(sh)
    dev_ms = [a.elapsed_time(b) for a, b in evs]
    smp.close()
    tiles = int(sum(news))
    per_tile = BYTES_PER_TILE[W] + W * W * 4        # elevation + normal tile, plus the synthetic residual written
    alg = tiles * per_tile
    gpu_s = sum(dev_ms) / 1000.0
    peak, src = hbm_peak()
    busy = [d for d, k in zip(dev_ms, news) if k > 0]
    return {"workload": "camera path of %d frames, 10 km -> 50 m, level 0-14 quadtree, %d-slot caches, "
                        "101x101 elevation + normal tiles, synthetic residuals, noise 300*0.55^l" % (frames, slots),
            "frames": frames, "new_tiles": tiles, "new_tiles_per_frame": {"mean": tiles / frames, "max": int(max(news)),
                                                                          "min": int(min(news))},
            "quadtree_tiles_per_frame": {"mean": float(np.mean([len(r) for r in reqs])),
                                         "max": int(max(len(r) for r in reqs))},
            "tiles_per_s": tiles / (total_ms / 1000.0),
            "frame_ms": {"p50": float(np.percentile(host_ms, 50)), "p99": float(np.percentile(host_ms, 99)),
                         "max": float(max(host_ms)), "mean": float(np.mean(host_ms))},
            "device_ms_per_frame": {"p50": float(np.percentile(dev_ms, 50)), "p99": float(np.percentile(dev_ms, 99)),
                                    "mean": float(np.mean(dev_ms))},
            "device_tiles_per_s": tiles / gpu_s if gpu_s > 0 else None,
            "request_generation_ms_per_frame": req_ms,
            "host_phases": phases,
            "algorithmic_bytes_per_tile": per_tile,
            "roofline": {"bound": "hbm", "achieved": alg / gpu_s / 1e9 if gpu_s > 0 else None, "peak": peak,
                         "unit": "GB/s", "frac": alg / gpu_s / 1e9 / peak if gpu_s > 0 else None, "peak_source": src,
                         "over": "device time of the frames' updates (CUDA events)",
                         "busy_frames_device_ms_p50": float(np.percentile(busy, 50)) if busy else None},
            "timing": "host clock per frame around tp_sampler_update + stream synchronisation; requests precomputed"}


def learned_section(tp, torch, stream, sh, args, plain_w101):
    """The learned-residual form beside the plain one.  Training data (seed S): the
    residual pyramid of a procedural 12-octave fBm sampled on 96 x 2^7 + 1 points
    (device preprocess; levels 1-7: 21,844 tile pairs, 174,752 with the 8
    symmetries) plus pairs at levels 6-12 sampled on the tiles' own windows of the
    same field (below the 12289^2 grid's resolution); Adam, batch 256.  Evaluation
    on terrain NOT trained on (seed S + 1000): levels 6-12 (the configuration's
    evaluation levels) and the held-out pyramid's levels 1-7, per level RMS / max
    height error and normal-angle error of the learned residuals against the plain
    method's (no residual).  Then the net's inference rate (tiles/s, tensor FLOP/s)
    and the rate of learned-form tiles (net + elevation kernel)."""
    from proland_gb300 import learned as L
    W, B = 101, 256
    deep_levels = list(range(6, 13))
    with torch.cuda.stream(stream):
        pyramid = L.build_pyramid(args.learned_levels, seed=args.seed)
        data = L.merge(pyramid, L.deep_pairs(deep_levels, args.learned_deep, seed=args.seed, tile_seed=args.seed))
        del pyramid
        si, so = L.level_sigmas(data)
        net = L.LearnedPredictor(W, B, seed=1)
        net.set_sigmas(si, so)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        losses = L.train(net, data, args.learned_steps, batch=args.learned_batch, lr=1e-3, lr_final=1e-4)
        torch.cuda.synchronize()
        train_ms = 1000.0 * (time.perf_counter() - t0) / max(1, args.learned_steps)
        held_seed = args.seed + 1000
        held = L.deep_pairs(deep_levels, 256, seed=held_seed, tile_seed=held_seed)
        ev = L.evaluate(net, held, so)
        held_pyr = L.build_pyramid(args.learned_levels, seed=held_seed)
        ev_pyr = L.evaluate(net, held_pyr, so)
        del held, held_pyr
        # inference: B tiles of level 6 per call, inputs resident
        idx = torch.arange(B, device="cuda") % data["up"].shape[0]
        up = data["up"].index_select(0, idx).contiguous()
        lv = [6] * B
        out = torch.empty_like(up)
        for _ in range(3):
            net.forward(up, lv, out=out)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 20
        e0.record(stream)
        for _ in range(reps):
            net.forward(up, lv, out=out)
        e1.record(stream)
        torch.cuda.synchronize()
        net.check()
        fwd_ms = e0.elapsed_time(e1) / reps
        # learned-form tiles: residuals predicted into slots, then the elevation kernel
        elev = tp.TileStorage(W, 3, B + 1)
        res = tp.TileStorage(W, 1, B)
        nrm = tp.TileStorage(W - 4, 2, B + 1)
        par = data["up"][0].cpu().numpy()[None]
        elev.upload(0, tp.ZF, par)
        elev.upload(0, tp.ZM, np.maximum(par, 0))
        jobs = [tp.make_job(6, 10 + (k % 2), 20 + (k // 2) % 2, out_slot=1 + k, parent_slot=0, residual_slot=k,
                            normal_slot=1 + k, tile_meters=50000.0 / 64) for k in range(B)]
        params = tp.make_params()
        for _ in range(3):
            net.predict_residuals(elev, jobs, res, sh)
            tp.elevation_batch(elev, res, nrm, params, jobs, sh)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            net.predict_residuals(elev, jobs, res, sh)
            tp.elevation_batch(elev, res, nrm, params, jobs, sh)
        stream.synchronize()
        form_ms = 1000.0 * (time.perf_counter() - t0) / reps
        tp.stream_check(sh)
    trained = (net.get_params(), si, so)
    used, executed = learned_flops(W)
    peak = None
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except (OSError, ValueError, KeyError):
        peak = 1900.0
    tflops = B * used / (fwd_ms / 1000.0) / 1e12
    net.close()
    return trained, {
        "tile_width": W, "batch": B,
        "net_tiles_per_s": B / (fwd_ms / 1000.0), "net_ms_per_batch": fwd_ms,
        "form_tiles_per_s": B / (form_ms / 1000.0), "form_ms_per_batch": form_ms,
        "plain_tiles_per_s_w101": plain_w101["tiles_per_s"] if plain_w101 else None,
        "tensor": {"achieved_tflops": tflops, "executed_tflops": B * executed / (fwd_ms / 1000.0) / 1e12,
                   "peak_tflops": peak, "frac": tflops / peak,
                   "flops_per_tile": used, "executed_flops_per_tile": executed},
        # each layer is a separate launch whose activations go through HBM: the forward
        # pass is bound by those bytes (64 B per pixel in and out of each hidden layer)
        "hbm": {"bytes_per_tile": learned_bytes(101),
                "achieved_gbs": B * learned_bytes(101) / (fwd_ms / 1000.0) / 1e9,
                "peak_gbs": hbm_peak()[0],
                "frac": B * learned_bytes(101) / (fwd_ms / 1000.0) / 1e9 / hbm_peak()[0]},
        "train": {"steps": args.learned_steps, "batch": args.learned_batch, "lr": "1e-3 decaying to 1e-4",
                  "optimizer": "Adam", "ms_per_step": train_ms,
                  "loss_first": float(np.mean(losses[:20])), "loss_last": float(np.mean(losses[-20:])),
                  "pairs": int(data["up"].shape[0]),
                  "data": "%d-level residual pyramid of a 12-octave fBm on %d^2 samples (device preprocess) plus "
                          "%d pairs per level at levels 6-12 on the tiles' own windows, seed %d, 8 symmetries"
                          % (args.learned_levels, 96 * (1 << args.learned_levels) + 1, args.learned_deep, args.seed)},
        "levels": {str(l): {k: (round(v, 7) if isinstance(v, float) else v) for k, v in e.items()}
                   for l, e in ev.items()},
        "levels_note": "held-out terrain (fBm seed %d), 256 tiles per level; sigma = RMS of the residual = the plain "
                       "method's RMS error; bar: rms_over_sigma <= 0.05" % (args.seed + 1000),
        "levels_meeting_5pct_bar": [int(l) for l, e in ev.items() if e["rms_over_sigma"] <= 0.05],
        "pyramid_levels": {str(l): {k: (round(v, 7) if isinstance(v, float) else v) for k, v in e.items()}
                           for l, e in ev_pyr.items()},
    }


def planet_section(tp, torch, stream, sh, args, trained):
    """Planet-scale mixed frames: requests on six cube faces, 197-wide tiles at levels
    0-16, stored residuals through level 10, residuals of the learned net (trained on
    101-wide tiles; the net is fully convolutional) at 11-16, sphere normals.  A step
    = learned residuals in chunks + one persistent elevation launch (CUDA graph) +
    the normal pass.  Errors per level against FP64 on sampled tiles."""
    import oracle
    from proland_gb300 import learned as L, planet
    params, si, so = trained
    pf = planet.PlanetFrame(n=args.planet_requests, seed=args.seed + 7)
    pf.allocate()
    net = L.LearnedPredictor(197, 512, seed=1)
    net.set_params(params)
    net.set_sigmas(si, so)
    with torch.cuda.stream(stream):
        pf.build(net, chunk=512)
        pf.frame.autotune(sh, repeats=3)
        for _ in range(2):
            pf.produce(sh)
        torch.cuda.synchronize()
        steps = 5
        parts = {"learned": 0.0, "elevation": 0.0, "normals": 0.0}
        t_all = time.perf_counter()
        for _ in range(steps):
            t0 = time.perf_counter()
            for arr in pf.learned_chunks:
                net.predict_residuals(pf.elev, arr, pf.res, sh)
            stream.synchronize()
            t1 = time.perf_counter()
            pf.frame.graph_launch(sh)
            stream.synchronize()
            t2 = time.perf_counter()
            tp.normal_batch(pf.elev, pf.nrm, pf.all_jobs_arr, pf.root, sh)
            stream.synchronize()
            t3 = time.perf_counter()
            parts["learned"] += t1 - t0
            parts["elevation"] += t2 - t1
            parts["normals"] += t3 - t2
        ms = 1000.0 * (time.perf_counter() - t_all) / steps
        tp.stream_check(sh)
    errs = pf.fp64_errors(oracle, per_level=2)
    out = {"requests": pf.n, "tile_width": 197, "levels": "0-16", "faces": 6,
           "learned_tiles": int(len(pf.learned_idx)), "stored_max_level": pf.stored_max,
           "tiles_per_s": pf.n / (ms / 1000.0), "ms_per_step": ms,
           "ms_learned": 1000.0 * parts["learned"] / steps, "ms_elevation": 1000.0 * parts["elevation"] / steps,
           "ms_normals": 1000.0 * parts["normals"] / steps, "elevation_shape": pf.frame.config(0),
           "timing": "host clock around each synchronised part, %d steps" % steps,
           "fp64_errors_per_level": {str(l): {k: (round(v, 8) if isinstance(v, float) else v) for k, v in e.items()}
                                     for l, e in errs.items()}}
    pf.close()
    net.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--requests", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default work-unit shapes")
    ap.add_argument("--no-per-width", action="store_true", help="skip the per-width timings")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-residual form")
    ap.add_argument("--learned-steps", type=int, default=3000, help="training steps before the learned timings")
    ap.add_argument("--learned-deep", type=int, default=2048,
                    help="training pairs per level at levels 6-12 sampled on the tiles' own windows")
    ap.add_argument("--learned-only", action="store_true", help="run the learned form alone and print its object")
    ap.add_argument("--learned-batch", type=int, default=256, help="training batch")
    ap.add_argument("--learned-levels", type=int, default=7,
                    help="levels of the training pyramid (7: 96 x 2^7 + 1 samples, 21,844 tile pairs)")
    ap.add_argument("--no-planet", action="store_true", help="skip the planet-scale mixed frame")
    ap.add_argument("--no-ortho", action="store_true", help="skip the ortho (colour) tile frame")
    ap.add_argument("--ortho-only", action="store_true",
                    help="run the ortho frame alone and print its object (for profiling)")
    ap.add_argument("--ortho-rgb", action="store_true", help="ortho frame with RGB instead of HSV noise")
    ap.add_argument("--planet-requests", type=int, default=16384)
    ap.add_argument("--no-layers", action="store_true", help="skip the elevation layer pass")
    ap.add_argument("--no-quadtree", action="store_true", help="skip the dependency-ordered quadtree frame")
    ap.add_argument("--no-streaming", action="store_true", help="skip the view-driven streaming frames")
    ap.add_argument("--frame-only", action="store_true",
                    help="the frame's device-resident launches alone (warm-up + steps), for profiling: prints "
                         "ms per step and the tiles of each width")
    ap.add_argument("--streaming-only", action="store_true",
                    help="run the view-driven streaming frames alone and print their object")
    ap.add_argument("--quadtree-only", action="store_true",
                    help="run the dependency-ordered quadtree frame alone and print its object")
    ap.add_argument("--layers-only", action="store_true",
                    help="run the elevation layer pass alone and print its object (for profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import proland_gb300 as tp

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    warmup = max(args.warmup, 3)

    from proland_gb300 import replicas
    if args.layers_only:
        stream = torch.cuda.Stream()
        print(json.dumps({"layers": layers_section(tp, torch, stream, C.c_void_p(stream.cuda_stream), args)}))
        return
    if args.learned_only:
        stream = torch.cuda.Stream()
        print(json.dumps({"learned": learned_section(tp, torch, stream, C.c_void_p(stream.cuda_stream), args, None)[1]}))
        return
    if args.streaming_only:
        stream = torch.cuda.Stream()
        print(json.dumps({"streaming": streaming_section(tp, torch, stream, C.c_void_p(stream.cuda_stream), args)}))
        return
    if args.quadtree_only:
        stream = torch.cuda.Stream()
        print(json.dumps({"quadtree": quadtree_section(tp, torch, stream, C.c_void_p(stream.cuda_stream), args)}))
        return
    if args.ortho_only:
        stream = torch.cuda.Stream()
        print(json.dumps({"ortho": ortho_section(tp, torch, stream, C.c_void_p(stream.cuda_stream), args)}))
        return
    classes = make_frame(args.requests, replicas.rank_seed(args.seed, rank), tp.noise_select)
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    params = tp.make_params()
    for fc in classes:
        fc.make_jobs(tp)
        fc.allocate(tp)
        fc.pin(torch)
        fc.upload_inputs(tp, sh)
        arr = (tp.TileJob * fc.n)(*fc.jobs)
        fc.dev_jobs = torch.empty(C.sizeof(arr), dtype=torch.uint8, device="cuda")
        fc.dev_jobs.copy_(torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8))
    torch.cuda.synchronize()

    # the whole frame (one persistent launch per tile width, the two overlapping), replayed from a CUDA graph
    frame = tp.Frame()
    for fc in classes:
        frame.add_device(fc.elev, fc.res, fc.nrm, params, C.c_void_p(fc.dev_jobs.data_ptr()), fc.n,
                         has_dependencies=False)

    if not args.no_autotune:
        frame.autotune(sh, repeats=5)
    tuned = {"W%d" % fc.W: frame.config(i) for i, fc in enumerate(classes)}
    if args.frame_only:
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                frame.graph_launch(sh)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            frame.graph_launch(sh)
        e1.record(stream)
        torch.cuda.synchronize()
        tp.stream_check(sh)
        print(json.dumps({"frame_only": {"ms_per_step": e0.elapsed_time(e1) / args.steps, "warmup": warmup,
                                         "steps": args.steps, "tiles": {"W%d" % fc.W: fc.n for fc in classes},
                                         "shapes": tuned}}))
        return

    def step(events=None):
        if events is not None:
            events[0][0].record(stream)
        frame.graph_launch(sh)
        if events is not None:
            events[0][1].record(stream)

    with torch.cuda.stream(stream):
        for _ in range(warmup):
            step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    kernel_ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))]
                 for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t_start.record(stream)
    for s in range(args.steps):
        step(kernel_ev[s])
    t_end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    tp.stream_check(sh)
    ms_total = t_start.elapsed_time(t_end)
    kernel_ms = sum(kernel_ev[s][0][0].elapsed_time(kernel_ev[s][0][1]) for s in range(args.steps)) / args.steps
    ms_total = replicas.max_over_ranks(ms_total, dist if world > 1 else None, "cuda")
    ms_step = ms_total / args.steps
    tiles = sum(fc.n for fc in classes)
    value = replicas.whole_job_rate(tiles, ms_step, world)

    # the same frame with the two launches one after the other, for comparison
    separate_ms = None
    if len(classes) == 2:
        frame.overlap_classes(False)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                frame.graph_launch(sh)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            frame.graph_launch(sh)
        e1.record(stream)
        torch.cuda.synchronize()
        tp.stream_check(sh)
        separate_ms = e0.elapsed_time(e1) / args.steps
        frame.overlap_classes(True)

    # per tile width: each width alone in its own frame, same tuned shape
    per_width = {}
    for fc in ([] if args.no_per_width else classes):
        fw = tp.Frame()
        fw.add_device(fc.elev, fc.res, fc.nrm, params, C.c_void_p(fc.dev_jobs.data_ptr()), fc.n,
                      has_dependencies=False)
        if not args.no_autotune:
            fw.autotune(sh, repeats=3)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                fw.graph_launch(sh)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            fw.graph_launch(sh)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        gbs = fc.n * BYTES_PER_TILE[fc.W] / (ms / 1000.0) / 1e9
        per_width["W%d" % fc.W] = {"tiles": fc.n, "ms": ms, "tiles_per_s": fc.n / (ms / 1000.0),
                                   "achieved_gbs": gbs, "frac": gbs / hbm_peak()[0], "shape": fw.config(0)}
        fw.close()
    tp.stream_check(sh)

    # end to end through the C ABI with host buffers: tp_elevation_batch_host per
    # tile width (chunked host->device copies, launches and device->host copies
    # overlapping), each width on its own caller stream
    e2e_ms = []
    pipes = [tp.HostPipeline(fc.W, chunk=E2E_CHUNK[fc.W]) for fc in classes] if args.e2e_steps > 0 else []
    e2e_streams = [torch.cuda.Stream() for _ in classes]
    for s in range(args.e2e_steps + 2 if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for fc, pipe, st in zip(classes, pipes, e2e_streams):
            fc.run_host(tp, pipe, params, C.c_void_p(st.cuda_stream))
        for st in e2e_streams:
            st.synchronize()
        if s >= 2:
            e2e_ms.append(1000.0 * (time.perf_counter() - t0))
    for st in e2e_streams:
        tp.stream_check(C.c_void_p(st.cuda_stream))
    e2e_check = check_host_outputs(classes) if pipes else None
    # the same frame returning zf and the normals only (zc, zm left on the device: the
    # reference's CPU producer fills zf only, and zm = max(zf, 0) is rebuilt on the host)
    e2e_min_ms = []
    for s in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for fc, pipe, st in zip(classes, pipes, e2e_streams):
            pipe.run(params, fc.jobs, fc.h_parent_zf, None, fc.h_residual, fc.h_zf, None, None, fc.h_nx, fc.h_ny,
                     C.c_void_p(st.cuda_stream))
        for st in e2e_streams:
            st.synchronize()
        if s >= 1:
            e2e_min_ms.append(1000.0 * (time.perf_counter() - t0))
    for st in e2e_streams:
        tp.stream_check(C.c_void_p(st.cuda_stream))
    for pipe in pipes:
        pipe.close()
    # the median step: the host link is shared with the box's other GPU, and a step that
    # meets another job's transfer takes several times longer (the mean is reported too)
    e2e_step = float(np.median(e2e_ms)) if e2e_ms else float("nan")
    e2e_step = replicas.max_over_ranks(e2e_step, dist if world > 1 else None, "cuda")

    if rank != 0:
        dist.barrier()
        dist.destroy_process_group()
        return

    peak, peak_src = hbm_peak()
    alg = {fc.W: fc.n * BYTES_PER_TILE[fc.W] for fc in classes}
    achieved = sum(alg.values()) / (kernel_ms / 1000.0) / 1e9
    # DRAM bytes of one step's launches (read + write): the per-tile traffic of a small
    # capture of the same kernel (profiles/frame_kernel_traffic.txt) times this frame's tiles
    pt = traffic_per_tile()
    traffic = sum(pt[fc.W] * fc.n for fc in classes) if pt and all(fc.W in pt for fc in classes) else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": frame_config(classes, world),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_src,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per tile of a 1024-request "
                                       "capture (profiles/frame_kernel_traffic.txt), times this frame's tiles",
                     "kernel": "frame_kernel (one persistent launch per tile width, the two on forked "
                               "streams of a CUDA graph)",
                     "kernel_ms": kernel_ms, "units_per_launch": frame.units(), "per_width": per_width,
                     "autotuned": tuned,
                     "serialised_launches_ms_per_step": separate_ms,
                     "algorithmic_bytes_per_step": sum(alg.values())},
        "e2e": {"value": world * tiles / (e2e_step / 1000.0), "unit": UNIT, "ms_per_step": e2e_step,
                "h2d_bytes_per_step": sum(fc.h2d_bytes for fc in classes),
                "d2h_bytes_per_step": sum(fc.d2h_bytes for fc in classes),
                "path": "tp_elevation_batch_host per tile width (chunks of %s tiles, copies overlapping launches)"
                        % "/".join(str(E2E_CHUNK[fc.W]) for fc in classes),
                "identical_to_device_run": e2e_check,
                "step_ms": {"min": min(e2e_ms), "median": float(np.median(e2e_ms)), "max": max(e2e_ms),
                            "mean": float(np.mean(e2e_ms)), "steps": len(e2e_ms)} if e2e_ms else None,
                "value_from": "median step",
                "planes": "zf, zc, zm, nx, ny",
                "zf_and_normals_only": {
                    "value": (world * tiles / (float(np.median(e2e_min_ms)) / 1000.0)) if e2e_min_ms else None,
                    "unit": UNIT, "ms_per_step": float(np.median(e2e_min_ms)) if e2e_min_ms else None,
                    "h2d_bytes_per_step": sum(fc.h2d_bytes for fc in classes),
                    "d2h_bytes_per_step": sum(fc.n * (fc.W * fc.W + 2 * (fc.W - 4) ** 2) * 4 for fc in classes),
                    "planes": "zf, nx, ny (zc, zm not copied back)"}},
        "gpu_launches": args.steps * len(classes),
        "clocks": clk,
        "max_err_vs_fp64": fp64_errors(tp, classes),
    }
    if not args.no_quadtree:
        line["quadtree"] = quadtree_section(tp, torch, stream, sh, args)
    if not args.no_streaming:
        line["streaming"] = streaming_section(tp, torch, stream, sh, args)
    if not args.no_ortho:
        line["ortho"] = ortho_section(tp, torch, stream, sh, args)
    if not args.no_layers:
        line["layers"] = layers_section(tp, torch, stream, sh, args)
    if not args.no_learned:
        trained, line["learned"] = learned_section(tp, torch, stream, sh, args, per_width.get("W101"))
        if not args.no_planet:
            line["planet"] = planet_section(tp, torch, stream, sh, args, trained)
    if not args.no_cpu:
        line["cpu_baseline"] = time_cpu(classes)
    print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""Benchmark of the b200 render path on one or more GB300s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

A step is one rendered frame of the workload into an accumulating
framebuffer.  Prints one JSON line (rank 0).  The headline workload is the
path tracer on the instanced displaced spheres at 1920x1080, 16 spp; with
N = 1 the same line also carries, under "configs", one object per other
measured configuration: the AO renderer (C0), the SciVis volume (C2), the
batched requests (C3) and the learned-cache study (C4: time to relMSE
<= 0.01 of the learned-cache path tracer against the plain one).

value      Mrays/s of all ranks: rays traced (counted by the kernels' stats
           pass over the same frames) / device time of the timed frames
           (CUDA events on the render stream; L2 flushed before every frame).
e2e        the same metric end to end through the public API with host
           buffers.  Path tracer: an OSPRay application's frame loop on
           libospray.so (ospRenderFrame + ospWait + ospMapFrameBuffer with
           the RGBA32F colour copied to host memory + ospUnmapFrameBuffer; the
           world is committed once, as an application does); the other
           workloads through the b200 C ABI (render call + b200_frame_read).
roofline   algorithmic bytes of the dominant kernel (traversal: 48 B ray
           record + 80 B per BVH node visit + 48 B per triangle and 20 B per
           sphere fetched) per launch / its CUDA-event launch time, against
           the measured HBM copy bandwidth; plus the issue activity, lanes
           per instruction and L2 throughput of a small-case ncu capture of
           the same kernel, which name the real limiter ("bound").
cpu_baseline  the CPU oracle (a restatement of the reference's ISPC path) on
           this machine's host cores, on a bounded, fixed sample of the same
           frames (row bands spread over the whole frame).
--impl reference  times that CPU implementation alone on the same sample,
           as the reference arm (the reference's ISPC+Embree device cannot be
           built here).

Multi-GPU: the render path does not exchange data between GPUs; N ranks
render N independent replicas ("replicas only"), scaling is weak.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 512 << 20

# DRAM traffic of the dominant kernel per algorithmic byte, from one ncu
# capture of a small case of the same kernel (dram__bytes_read.sum +
# dram__bytes_write.sum of the captured launches / their algorithmic bytes);
# the summaries under profiles/ give the commands.  Scaled to the bench's
# launches by their algorithmic bytes.
TRAFFIC = {
    "pt_instanced_spheres_1080p": {"dram_per_alg_byte": 0.098,
                                   "source": "profiles/k_trace_queue_pt_instanced_480x270_limiter.md"},
    "scivis_volume_512cube_1024": {"dram_per_alg_byte": 0.21,
                                   "source": "profiles/k_render_scivis_volume_512cube.md"},
}

# What limits the dominant kernel, from the same small-case ncu captures:
# issue activity (smsp__issue_active), active lanes per warp instruction
# (smsp__thread_inst_executed_per_inst_executed), L2 throughput
# (lts__t_bytes per second) per instantiation.
LIMITER = {
    "pt_instanced_spheres_1080p": {
        "bound": "issue",
        "issue_active": {"closest": 0.667, "shadow": 0.745},
        "lanes_per_instruction": {"closest": 14.59, "shadow": 10.39},
        "l2_gbs": {"closest": 1052.0, "shadow": 1576.0},
        "source": "profiles/k_trace_queue_pt_instanced_480x270_limiter.md"},
    "scivis_volume_512cube_1024": {
        "bound": "latency",
        "source": "profiles/k_render_scivis_volume_512cube.md"},
    "ao_heightfield_512": {
        "bound": "latency",
        "source": "profiles/k_render_ao_heightfield_512.md"},
}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 8:
                    continue
                try:
                    sm.append(float(f[0]))
                    mx.append(float(f[1]))
                except ValueError:
                    continue
                for n, v in zip(names, f[4:8]):
                    if v.lower() == "active":
                        reasons.add(n)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def _sig(x, digits=4):
    """x to `digits` significant figures (relMSE values span many decades)."""
    return float("%.*g" % (digits, x))


# --------------------------------------------------------------------------- workloads


class AOWorkload:
    """AO renderer, aoSamples 1, aoDistance 1e20, 512x512 RGBA32F, 1 spp, on
    the 256x256 height field (130,050 triangles) + 1,000 spheres (seed 0)."""
    name = "ao_heightfield_512"
    metric = "Mrays/s"

    def __init__(self, w=512, h=512):
        from ospray_gb300 import scenes
        self.w, self.h = w, h
        self.data = scenes.ao_heightfield_scene()
        self.config = {"workload": self.name, "renderer": "ao", "width": w, "height": h, "spp": 1,
                       "aoSamples": 1, "triangles": int(len(self.data["index"])),
                       "spheres": int(len(self.data["spheres"])), "pixelFilter": "gauss"}

    def setup(self, og, dev):
        from ospray_gb300 import scenes
        self.og = og
        t0 = time.perf_counter()
        self.scene = og.Scene(dev)
        scenes.build_ao_scene(self.scene, self.data)
        self.build_ms = (time.perf_counter() - t0) * 1e3
        c = self.data["camera"]
        self.cam = og.camera_desc(c["position"], c["direction"], c["up"], aspect=self.w / self.h)
        self.params = og.ao_params(spp=1, ao_samples=1, pixel_filter=og.PF_GAUSS)
        self.sparams = og.ao_params(spp=1, ao_samples=1, pixel_filter=og.PF_GAUSS, stats=True)
        self.fb = og.Frame(dev, self.w, self.h, og.FB_COLOR | og.FB_DEPTH | og.FB_ACCUM)
        self.color = np.empty((self.h, self.w, 4), np.float32)

    def step(self, stats=False):
        self.og.render_ao(self.scene, self.cam, self.sparams if stats else self.params, self.fb)

    def e2e_step(self):
        # parameters travel host->device with the launch; colour comes back
        self.og.render_ao(self.scene, self.cam, self.params, self.fb)
        self.og.lib().b200_frame_read(self.fb._h, self.og.FB_COLOR, self.color.ctypes.data, self.color.nbytes)
        return 40 + 52, self.color.nbytes

    def reset(self):
        self.fb.reset()

    def counters(self, reset=False):
        return self.scene.counters(reset)

    def cpu_frames(self, budget_s, nthreads):
        """Oracle frames on the host cores until budget_s: (rays, seconds, frames)."""
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle
        from ospray_gb300 import scenes
        o = oracle.Scene()
        scenes.build_ao_scene(o, self.data)
        c = self.data["camera"]
        cam = oracle.camera(c["position"], c["direction"], c["up"], aspect=self.w / self.h)
        oracle.lib().or_ray_count.restype = __import__("ctypes").c_uint64
        oracle.lib().or_ray_count(1)
        t0 = time.perf_counter()
        frames = 0
        while True:
            oracle.render_ao(o, cam, 2, self.w, self.h, frames=1, nthreads=nthreads)
            frames += 1
            if time.perf_counter() - t0 >= budget_s or frames >= 2000:
                break
        dt = time.perf_counter() - t0
        return int(oracle.lib().or_ray_count(1)), dt, frames


class PTWorkload:
    """Path tracer, 1920x1080, 16 spp, maxPathLength 5, Russian roulette from
    depth 3, on 64 instances of a 32,768-triangle displaced sphere (2.1 M
    triangles instanced) over a ground quad; principled materials; one 2x2
    quad light (intensity 20) and an ambient light (0.1)."""
    name = "pt_instanced_spheres_1080p"
    metric = "Mrays/s"

    def __init__(self, w=1920, h=1080, spp=16, seed=1, count=64, levels=6):
        from ospray_gb300 import scenes
        self.w, self.h, self.spp = w, h, spp
        self.data = scenes.pt_instanced_scene(seed=seed, count=count, levels=levels, width=w, height=h)
        self.config = {"workload": self.name, "renderer": "pathtracer", "width": w, "height": h, "spp": spp,
                       "maxPathLength": 5, "roulettePathLength": 3, "instances": len(self.data["xfm"]),
                       "triangles_per_instance": int(len(self.data["index"])),
                       "triangles_instanced": int(len(self.data["index"]) * len(self.data["xfm"]) + 2),
                       "lights": "quad 2x2 intensity 20 + ambient 0.1", "pixelFilter": "gauss"}

    def setup(self, og, dev):
        from ospray_gb300 import scenes
        self.og = og
        t0 = time.perf_counter()
        self.scene = og.Scene(dev)
        scenes.build_pt_scene(self.scene, self.data)
        lights = []
        for L in self.data["lights"]:
            if L["type"] == "quad":
                lights.append(og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]))
            else:
                lights.append(og.ambient_light(L["intensity"]))
        self.scene.set_lights(lights)
        self.build_ms = (time.perf_counter() - t0) * 1e3
        c = self.data["camera"]
        self.cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
        self.params = og.pt_params(spp=self.spp, max_path_length=5, roulette_path_length=3)
        self.sparams = og.pt_params(spp=self.spp, max_path_length=5, roulette_path_length=3, stats=True)
        self.mats = og.materials_array(self.data["materials"])
        self.fb = og.Frame(dev, self.w, self.h, og.FB_COLOR | og.FB_DEPTH | og.FB_ACCUM)
        self.color = np.empty((self.h, self.w, 4), np.float32)
        self.dev = dev

    def step(self, stats=False):
        self.og.render_pt(self.scene, self.cam, self.sparams if stats else self.params, self.mats, self.fb)

    def image_stats(self, ref_spp):
        """Image statistics of one benchmark frame (frame 0, spp samples per
        pixel) against a ref_spp-sample render of the same scene on the GPU:
        relMSE over the frame; over the CPU baseline's bands the GPU's and the
        CPU oracle's relMSE and mean, with the mean's standard error (the
        CPU bands render the same frame 0 samples)."""
        og = self.og
        self.fb.reset()
        self.step()
        ref = og.Frame(self.dev, self.w, self.h, og.FB_COLOR | og.FB_ACCUM)
        for _ in range(max(1, ref_spp // self.spp)):
            og.render_pt(self.scene, self.cam, self.params, self.mats, ref)
        out = {"reference_spp": int(max(1, ref_spp // self.spp) * self.spp), "frame_spp": self.spp,
               "relmse_gpu": _sig(og.relmse(self.fb, ref))}
        cpu = getattr(self, "cpu_color", None)
        if cpu is not None:
            r = ref.read(og.FB_ACCUM)[..., :3]
            g = self.fb.read(og.FB_ACCUM)[..., :3]
            rows = np.concatenate([np.arange(a, b) for a, b in self.cpu_bands()])

            def rel(x):
                return float(np.mean((x[rows] - r[rows]) ** 2 / (r[rows] ** 2 + 0.01)))
            c = cpu[..., :3]
            d = (g[rows] - c[rows]).reshape(-1)
            out.update({"bands_relmse_gpu": _sig(rel(g)), "bands_relmse_cpu": _sig(rel(c)),
                        "bands_mean_gpu": round(float(g[rows].mean()), 6),
                        "bands_mean_cpu": round(float(c[rows].mean()), 6),
                        "bands_mean_diff_se": round(float(d.std() / np.sqrt(d.size)), 8)})
        self.fb.reset()
        return out

    def e2e_setup(self):
        """The same workload built by an OSPRay application on libospray.so."""
        from ospray_gb300 import osp
        if getattr(self, "app", None) is None:
            L = osp.lib()
            if L.ospInit(None, None) != 0:
                raise RuntimeError("ospInit: %s" % L.ospDeviceGetLastErrorMsg(None))
            self.app = osp.PathTracerApp(self.data, self.spp, 5, 3, self.w, self.h)
        self.app.reset()

    def e2e_step(self):
        return self.app.frame()

    e2e_api = "libospray.so: ospRenderFrame + ospWait + ospMapFrameBuffer (RGBA32F colour to host) + ospUnmapFrameBuffer"

    def reset(self):
        self.fb.reset()

    def counters(self, reset=False):
        return self.scene.counters(reset)

    def cpu_bands(self, nbands=12, rows=8):
        """A fixed sample of the frame: `nbands` bands of `rows` rows centred on
        evenly spaced heights, so the sample sees the whole frame's content."""
        out = []
        for i in range(nbands):
            c = int((i + 0.5) * self.h / nbands)
            out.append((max(0, c - rows // 2), min(self.h, c + rows // 2)))
        return out

    def cpu_frames(self, budget_s, nthreads, passes=None):
        """Oracle passes over the fixed band sample until budget_s (or
        `passes` passes): (rays, seconds, passes)."""
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle
        from ospray_gb300 import scenes
        if not hasattr(self, "_orc"):
            o = oracle.Scene()
            scenes.build_pt_scene(o, self.data)
            self._orc = (o, oracle.PtWorld(self.data["materials"], self.data["lights"]))
            c = self.data["camera"]
            self._ocam = oracle.camera(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
            self._op = oracle.pt_params(spp=self.spp, max_path_length=5, roulette_path_length=3)
            oracle.render_pt(o, self._orc[1], self._ocam, oracle.pt_params(spp=1), 4, 4)  # albedo tables
        o, ow = self._orc
        bands = self.cpu_bands()
        oracle.lib().or_ray_count(1)
        t0 = time.perf_counter()
        n = 0
        color = np.zeros((self.h, self.w, 4), np.float32)
        while True:
            for y0, y1 in bands:
                img = oracle.render_pt(o, ow, self._ocam, self._op, self.w, self.h, rows=(y0, y1), nthreads=nthreads)
                color[y0:y1] = img["color"][y0:y1]
            n += 1
            self.cpu_color = color
            dt = time.perf_counter() - t0
            if (passes is not None and n >= passes) or (passes is None and dt >= budget_s):
                break
        rays = int(oracle.lib().or_ray_count(1))
        nrows = sum(b - a for a, b in bands)
        self.cpu_sample = "%d bands of 8 rows spread over the frame (%d of %d rows) x %d px x %d spp, %d pass(es)" % (
            len(bands), nrows, self.h, self.w, self.spp, n)
        return rays, dt, n


class ScivisWorkload:
    """SciVis volume rendering: 512^3 float32 fractal-noise volume through a
    256-entry transfer function, volumeSamplingRate 1, 1024x1024, 4 spp,
    orbit camera.  Unit: volume samples (Msamples/s)."""
    name = "scivis_volume_512cube_1024"
    metric = "Msamples/s"
    launches_per_frame = 2  # march + post-process (colour conversion)

    def __init__(self, w=1024, h=1024, n=512, spp=4):
        from ospray_gb300 import scenes
        self.w, self.h, self.spp = w, h, spp
        self.data = scenes.volume_scene(n=n, width=w, height=h)
        self.config = {"workload": self.name, "renderer": "scivis", "width": w, "height": h, "spp": spp,
                       "volume": "%d^3 float32" % n, "volumeSamplingRate": 1.0, "transfer_function": 256,
                       "shadows": True, "lights": "none (shadows inert)", "pixelFilter": "gauss"}

    def setup(self, og, dev):
        self.og = og
        d = self.data
        t0 = time.perf_counter()
        self.scene = og.Scene(dev)
        self.scene.set_volume(d["volume"], d["origin"], d["spacing"], d["color"], d["opacity"], d["value_range"])
        self.build_ms = (time.perf_counter() - t0) * 1e3
        c = d["camera"]
        self.cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
        # shadows on as the configuration names them; the world has no lights, so they cast nothing
        self.params = og.scivis_params(spp=self.spp, shadows=True)
        self.sparams = og.scivis_params(spp=self.spp, shadows=True, stats=True)
        self.fb = og.Frame(dev, self.w, self.h, og.FB_COLOR | og.FB_ACCUM)
        self.color = np.empty((self.h, self.w, 4), np.float32)

    def step(self, stats=False):
        self.og.render_scivis(self.scene, self.cam, self.sparams if stats else self.params, self.fb)

    def e2e_step(self):
        self.og.render_scivis(self.scene, self.cam, self.params, self.fb)
        self.og.lib().b200_frame_read(self.fb._h, self.og.FB_COLOR, self.color.ctypes.data, self.color.nbytes)
        return 40 + 32, self.color.nbytes

    def reset(self):
        self.fb.reset()

    def counters(self, reset=False):
        c = self.scene.counters(reset)
        return c

    def units(self, c):
        return int(c[1])  # volume samples

    def bytes_per_unit(self):
        return 32.0

    def cpu_frames(self, budget_s, nthreads, passes=None):
        """Oracle passes over 8 bands of 4 rows spread over the frame."""
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle
        d = self.data
        if not hasattr(self, "_orc"):
            self._orc = oracle.VolumeModel(d["volume"], d["origin"], d["spacing"], d["color"], d["opacity"],
                                           d["value_range"])
            c = d["camera"]
            self._ocam = oracle.camera(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
        bands = [(int((i + 0.5) * self.h / 8) - 2, int((i + 0.5) * self.h / 8) + 2) for i in range(8)]
        oracle.lib().or_volume_sample_count(1)
        t0 = time.perf_counter()
        n = 0
        while True:
            for y0, y1 in bands:
                oracle.render_scivis_volume(self._orc, self._ocam, 2, self.w, self.h, spp=self.spp, rows=(y0, y1),
                                            nthreads=nthreads)
            n += 1
            dt = time.perf_counter() - t0
            if (passes is not None and n >= passes) or (passes is None and dt >= budget_s):
                break
        samples = int(oracle.lib().or_volume_sample_count(1))
        self.cpu_sample = "8 bands of 4 rows spread over the frame x %d px x %d spp, %d pass(es)" % (
            self.w, self.spp, n)
        return samples, dt, n


class BatchWorkload:
    """Batched serving: 64 requests (resolution uniform over 256^2, 512^2,
    768^2, 1024^2, 1280x720; spp uniform in 1..8; AO or path tracer with
    probability 1/2; each on its own seeded height field of 65k-1M triangles
    plus 1,000 spheres) rendered as one batched wavefront per step: the
    wavefront kernels replayed as a CUDA graph (mode "graph") or one
    cooperative persistent launch (mode "persistent"), launch shape chosen by
    the autotuner at setup.  Reports aggregate Mrays/s, and per-request
    latency (p50/p99 of completion times after the render starts) of the
    batch and of the same requests rendered one after another with
    single-request calls."""
    name = "batch_64_requests"
    metric = "Mrays/s"
    mode = "graph"

    def __init__(self, count=64, seed=0):
        from ospray_gb300 import scenes
        self.reqs = scenes.batch_requests(seed, count)
        kinds = [r["renderer"] for r in self.reqs]
        self.config = {"workload": self.name, "requests": count, "seed": seed,
                       "ao_requests": kinds.count("ao"), "pt_requests": kinds.count("pathtracer"),
                       "pixels": int(sum(r["width"] * r["height"] for r in self.reqs)),
                       "paths": int(sum(r["width"] * r["height"] * r["spp"] for r in self.reqs)),
                       "pt_params": "maxPathLength 20, roulettePathLength 5 (defaults)",
                       "ao_params": "aoSamples 1, aoDistance 1e20", "pixelFilter": "gauss"}

    def setup(self, og, dev):
        from ospray_gb300 import scenes
        self.og, self.dev = og, dev
        t0 = time.perf_counter()
        self.items = []
        tris = 0
        for r in self.reqs:
            sc = og.Scene(dev)
            tris += scenes.build_batch_request_scene(sc, r)
            c = dict(position=(0.5, 2.0, -1.5), direction=(0.0, -2.0, 2.0), up=(0.0, 1.0, 0.0))
            cam = og.camera_desc(c["position"], c["direction"], c["up"], aspect=r["width"] / r["height"])
            if r["renderer"] == "ao":
                p = og.ao_params(spp=r["spp"], ao_samples=1, pixel_filter=og.PF_GAUSS)
                sp = og.ao_params(spp=r["spp"], ao_samples=1, pixel_filter=og.PF_GAUSS, stats=True)
                mats = None
            else:
                p = og.pt_params(spp=r["spp"])
                sp = og.pt_params(spp=r["spp"], stats=True)
                mats = og.materials_array([r["material"]])
            fb = og.Frame(dev, r["width"], r["height"], og.FB_COLOR | og.FB_DEPTH | og.FB_ACCUM)
            seq = og.Frame(dev, r["width"], r["height"], og.FB_COLOR | og.FB_DEPTH | og.FB_ACCUM)
            self.items.append(dict(req=r, scene=sc, cam=cam, params=p, sparams=sp, mats=mats, fb=fb, seq=seq))
        self.config["triangles_total"] = int(tris)
        self.build_ms = (time.perf_counter() - t0) * 1e3
        self.batch = og.Batch(dev)
        for it in self.items:
            if it["req"]["renderer"] == "ao":
                self.batch.add_ao(it["scene"], it["cam"], it["params"], it["fb"])
            else:
                self.batch.add_pt(it["scene"], it["cam"], it["params"], it["mats"], it["fb"])
        # traversal statistics per ray from one single-request stats frame of each request
        rays = nodes = tri = sph = 0
        for it in self.items:
            self._single(it, stats=True)
            c = it["scene"].counters(reset=True)
            rays, nodes, tri, sph = rays + c[0], nodes + c[1], tri + c[2], sph + c[3]
        self.per_ray = (nodes / max(rays, 1), tri / max(rays, 1), sph / max(rays, 1))
        self.set_mode(self.mode)
        self.fb = self.items[0]["fb"]
        self.colors = [np.empty((it["req"]["height"], it["req"]["width"], 4), np.float32) for it in self.items]
        self._rays = 0

    def _mode(self):
        return self.og.BATCH_PERSISTENT if self.mode == "persistent" else self.og.BATCH_GRAPH

    def set_mode(self, mode):
        """Switches the batch's launch mode and autotunes for it (the
        persistent launch tunes the wave size only)."""
        self.mode = mode
        self.batch.render(mode=self._mode())  # the mode the autotuner tunes for
        t1 = time.perf_counter()
        best = self.batch.autotune(candidates=int(os.environ.get("B200_BATCH_TUNE_CANDIDATES", "6")))
        self.batch.render(mode=self._mode())
        self.config["mode"] = mode
        self.config["plan"] = self.batch.info()
        self.config["autotune"] = {"wavePaths": int(best.wavePaths), "traceBlocksPerSM": best.traceBlocksPerSM,
                                   "shadeBlocksPerSM": best.shadeBlocksPerSM,
                                   "seconds": round(time.perf_counter() - t1, 2)}
        if mode == "persistent":  # one grid of every co-resident block
            del self.config["autotune"]["traceBlocksPerSM"], self.config["autotune"]["shadeBlocksPerSM"]

    def kernels_per_frame(self):
        return self.batch.info()["kernels"]

    def _single(self, it, stats=False, seq=True):
        fb = it["seq"] if seq else it["fb"]
        p = it["sparams"] if stats else it["params"]
        if it["req"]["renderer"] == "ao":
            self.og.render_ao(it["scene"], it["cam"], p, fb)
        else:
            self.og.render_pt(it["scene"], it["cam"], p, it["mats"], fb)

    def step(self, stats=False):
        self.batch.render(mode=self._mode())
        if stats:
            self._rays += self.batch.timings()[1]

    def e2e_step(self):
        self.batch.render(mode=self._mode())
        d2h = 0
        for it, col in zip(self.items, self.colors):
            self.og.lib().b200_frame_read(it["fb"]._h, self.og.FB_COLOR, col.ctypes.data, col.nbytes)
            d2h += col.nbytes
        return 116 * len(self.items), d2h

    def reset(self):
        for it in self.items:
            it["fb"].reset()

    def counters(self, reset=False):
        r = self._rays
        if reset:
            self._rays = 0
        n, t, s = self.per_ray
        return [r, int(r * n), int(r * t), int(r * s)]

    def latency(self):
        """p50/p99 request completion (ms after the render starts): batch vs sequential."""
        og, dev = self.og, self.dev
        self.batch.render(mode=self._mode())
        bms, brays = self.batch.timings()
        for it in self.items:  # warm
            it["seq"].reset()
        dev.sync()
        e0 = dev.record_event()
        evs = []
        for it in self.items:
            self._single(it)
            evs.append(dev.record_event())
        dev.sync()
        sms = np.array([dev.event_ms(e0, e) for e in evs])
        for e in [e0] + evs:
            dev.release_event(e)

        def pct(a):
            return {"p50_ms": round(float(np.percentile(a, 50)), 3), "p99_ms": round(float(np.percentile(a, 99)), 3),
                    "makespan_ms": round(float(np.max(a)), 3)}
        return {"batched": pct(bms), "sequential": pct(sms),
                "sequential_mrays_s": round(brays / (float(np.max(sms)) * 1e-3) / 1e6, 3),
                "note": "completion time of each request after the render begins; sequential = the same "
                        "requests through b200_render_ao / b200_render_pt one after another"}

    def cpu_frames(self, budget_s, nthreads):
        """Oracle on the requests in order (AO whole frames, path tracing on a
        band of 16 centre rows), timing rendering only, until budget_s."""
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle
        from ospray_gb300 import scenes
        rays = 0
        dt = 0.0
        done = []
        for r in self.reqs:
            o = oracle.Scene()
            scenes.build_batch_request_scene(o, r, lights=False)
            c = dict(position=(0.5, 2.0, -1.5), direction=(0.0, -2.0, 2.0), up=(0.0, 1.0, 0.0))
            cam = oracle.camera(c["position"], c["direction"], c["up"], aspect=r["width"] / r["height"])
            oracle.lib().or_ray_count(1)
            t0 = time.perf_counter()
            if r["renderer"] == "ao":
                oracle.render_ao(o, cam, 2, r["width"], r["height"], spp=r["spp"], nthreads=nthreads)
                done.append("ao %dx%d" % (r["width"], r["height"]))
            else:
                world = oracle.PtWorld([r["material"]], [
                    dict(type="quad", position=(0.3, 1.2, 0.3), edge1=(0.4, 0, 0), edge2=(0, 0, 0.4),
                         intensity=20.0), dict(type="ambient", intensity=0.2)])
                y0 = r["height"] // 2 - 8
                oracle.render_pt(o, world, cam, oracle.pt_params(spp=r["spp"]), r["width"], r["height"],
                                 rows=(y0, y0 + 16), nthreads=nthreads)
                done.append("pt 16 rows of %dx%d" % (r["width"], r["height"]))
            dt += time.perf_counter() - t0
            rays += int(oracle.lib().or_ray_count(1))
            if dt >= budget_s:
                break
        self.cpu_sample = "first %d requests in order (%s)" % (len(done), ", ".join(done[:4]) + ", ...")
        return rays, dt, len(done)


AOWorkload.launches_per_frame = 2  # render + post-process (colour conversion)
AOWorkload.timed_kernels = ("ao",)
AOWorkload.roofline_kernel = "k_render_ao (camera + AO rays, one launch per frame)"
AOWorkload.e2e_api = "b200 C ABI: b200_render_ao + b200_frame_read (RGBA32F colour to host)"
PTWorkload.timed_kernels = ("trace_closest", "trace_shadow")
PTWorkload.roofline_kernel = "k_trace_queue (closest-hit and shadow instantiations)"
ScivisWorkload.timed_kernels = ("scivis",)
ScivisWorkload.roofline_kernel = "k_render_scivis_volume"
ScivisWorkload.e2e_api = "b200 C ABI: b200_render_scivis + b200_frame_read (RGBA32F colour to host)"
# generate, finalize, post-process, 6 bounces x (reset, trace, shade, shadow), queue partitions of bounces 1-5
PTWorkload.launches_per_frame = 3 + 6 * 4 + 5
BatchWorkload.launches_per_frame = None  # taken from the batch plan (b200_batch_info)
BatchWorkload.e2e_api = ("b200 C ABI: b200_batch_render (graph replay of the wavefront kernels, or the one "
                         "persistent launch) + b200_frame_read of every request")
WORKLOADS = {"ao": AOWorkload, "pt": PTWorkload, "scivis": ScivisWorkload, "batch": BatchWorkload}


# --------------------------------------------------------------------------- arms


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args):
    """The reference arm: the CPU implementation of the path on the host
    cores, each step one pass over the workload's fixed CPU sample."""
    ws, rank, local = dist_setup(args)
    if rank != 0:
        return
    wl = WORKLOADS[args.workload]()
    nthreads = os.cpu_count() or 1
    per_step = []
    rays_total = 0
    for i in range(args.warmup + args.steps):
        if hasattr(wl, "cpu_bands") or isinstance(wl, ScivisWorkload):
            rays, dt, _ = wl.cpu_frames(0.0, nthreads, passes=1)
        else:
            rays, dt, _ = wl.cpu_frames(args.cpu_budget / max(1, args.steps), nthreads)
        if i >= args.warmup:
            per_step.append((rays, dt))
            rays_total += rays
    secs = sum(dt for _, dt in per_step)
    value = rays_total / secs / 1e6
    line = {"metric": wl.metric, "value": round(value, 3), "unit": wl.metric, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(secs / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generators)", "config": wl.config, "impl": "reference",
            "cpu_baseline": {"value": round(value, 3), "unit": wl.metric, "cores": nthreads, "kind": "port",
                             "sample": "%s per step" % getattr(wl, "cpu_sample", "whole frames")},
            "e2e": {"value": round(value, 3), "unit": wl.metric, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measure(wl, args, og, dev, local, ws, cpu_budget):
    """Times `args.steps` frames of a set-up workload: device value, e2e,
    roofline of the dominant kernel, clocks, and (cpu_budget > 0) the CPU
    baseline.  Returns the JSON line as a dict (rank 0) or None."""
    import torch
    rank = int(os.environ.get("RANK", "0"))
    stream = torch.cuda.ExternalStream(dev.stream, device=torch.device("cuda", local))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=torch.device("cuda", local))
    wl.reset()
    for _ in range(args.warmup):
        wl.step()
    dev.sync()
    first_timed = wl.fb.frame_id
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(local)
    dev.sync()
    timed_kernels = getattr(wl, "timed_kernels", None)
    if timed_kernels:
        dev.kernel_timing(True)
        dev.kernel_times(reset=True)
    with Clocks(local) as clk:
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                evs[i][0].record(stream)
            wl.step()
            with torch.cuda.stream(stream):
                evs[i][1].record(stream)
        dev.sync()
        torch.cuda.synchronize(local)
    ktimes = None
    if timed_kernels:
        ktimes = dev.kernel_times(reset=True)
        dev.kernel_timing(False)
    if ws > 1:
        torch.distributed.barrier()
    times = [a.elapsed_time(b) for a, b in evs]
    dev_ms = float(sum(times))
    del flush
    # rays of exactly the timed frames: replay the same frame sequence in stats mode
    wl.reset()
    for _ in range(first_timed):
        wl.step()
    wl.counters(reset=True)
    for _ in range(args.steps):
        wl.step(stats=True)
    c = wl.counters(reset=True)
    rays, nodes, tris, sph = (int(x) for x in c)
    units = wl.units(c) if hasattr(wl, "units") else rays
    # end to end through the public API with host buffers
    if hasattr(wl, "e2e_setup"):
        wl.e2e_setup()
    else:
        wl.reset()
    for _ in range(2):
        wl.e2e_step()
    dev.sync()
    t0 = time.perf_counter()
    h2d = d2h = 0
    for _ in range(args.steps):
        h2d, d2h = wl.e2e_step()
    dev.sync()
    e2e_s = time.perf_counter() - t0

    local_vals = torch.tensor([dev_ms, e2e_s, float(units)], dtype=torch.float64, device=torch.device("cuda", local))
    if ws > 1:
        mx = local_vals.clone()
        torch.distributed.all_reduce(mx, op=torch.distributed.ReduceOp.MAX)
        sm = local_vals.clone()
        torch.distributed.all_reduce(sm, op=torch.distributed.ReduceOp.SUM)
        dev_ms_max, e2e_max, units_all = float(mx[0]), float(mx[1]), float(sm[2])
    else:
        dev_ms_max, e2e_max, units_all = dev_ms, e2e_s, float(units)
    if rank != 0:
        return None
    value = units_all / (dev_ms_max * 1e-3) / 1e6
    e2e_val = units_all / e2e_max / 1e6
    if hasattr(wl, "bytes_per_unit"):
        alg_bytes = wl.bytes_per_unit() * units
        note = "algorithmic volume bytes (32 B per trilinear sample)"
    else:
        alg_bytes = 48.0 * rays + 80.0 * nodes + 48.0 * tris + 20.0 * sph
        note = "algorithmic traversal bytes (48 B ray record + 80 B per node visit + 48 B per triangle, 20 B per sphere)"
    peak, kind = peaks()
    if ktimes:
        # the dominant kernel, timed live with CUDA events around its launches
        kms = sum(ktimes[k][0] for k in timed_kernels)
        klaunches = sum(ktimes[k][1] for k in timed_kernels)
        achieved = alg_bytes / (kms * 1e-3) / 1e9
        per_launch = alg_bytes / max(klaunches, 1)
        roof_kernel = {"kernel": wl.roofline_kernel, "launches": klaunches, "ms": round(kms, 3),
                       "share_of_step": round(kms / dev_ms, 4), "bytes_per_launch": round(per_launch)}
        note += " of the timed launches / their summed CUDA-event time"
    else:
        achieved = alg_bytes / (dev_ms * 1e-3) / 1e9
        per_launch = None
        roof_kernel = {"kernel": "whole step (launches captured in a CUDA graph)"}
        note += " per step / step time"
    traffic = None
    tp = TRAFFIC.get(wl.name)
    if tp and per_launch is not None:
        # ncu dram bytes per algorithmic byte of the same kernel, scaled to this launch size
        traffic = round(tp["dram_per_alg_byte"] * per_launch)
        note += "; traffic from %s" % tp["source"]
    lim = LIMITER.get(wl.name, {})
    roof = {"bound": lim.get("bound", "hbm"), "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic,
            "note": "%s; peak %s (%s)" % (note, kind, "of measured" if kind == "measured" else "of fallback")}
    for k in ("issue_active", "lanes_per_instruction", "l2_gbs"):
        if k in lim:
            roof[k] = lim[k]
    if "source" in lim:
        roof["limiter_source"] = lim["source"]
    roof.update(roof_kernel)
    line = {"metric": wl.metric, "value": round(value, 3), "unit": wl.metric, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dev_ms_max / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generators)",
            "config": dict(wl.config, l2="flushed before every frame (512 MiB write)",
                           parallelism="replicas" if ws > 1 else "single", build_ms=round(wl.build_ms, 2),
                           rays_per_frame=rays / args.steps, node_visits_per_ray=round(nodes / max(rays, 1), 3),
                           tri_tests_per_ray=round(tris / max(rays, 1), 3)),
            "e2e": {"value": round(e2e_val, 3), "unit": wl.metric, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "api": getattr(wl, "e2e_api", "b200 C ABI")},
            "gpu_launches": args.steps * (wl.launches_per_frame or wl.kernels_per_frame()),
            "roofline": roof,
            "clocks": clk.summary()}
    if hasattr(wl, "latency"):
        line["latency"] = wl.latency()
    if cpu_budget > 0:
        nthreads = os.cpu_count() or 1
        crays, cdt, _ = wl.cpu_frames(cpu_budget, nthreads)
        sample = getattr(wl, "cpu_sample", "frames of the same workload")
        line["cpu_baseline"] = {"value": round(crays / cdt / 1e6, 3), "unit": wl.metric, "cores": nthreads,
                                "kind": "port", "sample": "%s (%.1f s)" % (sample, cdt)}
    return line


def run_ours(args):
    import torch
    import ospray_gb300 as og
    ws, rank, local = dist_setup(args)
    if ws > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
    dev = og.Device(local)
    wl = WORKLOADS[args.workload]()
    if args.workload == "batch":
        wl.mode = args.batch_mode
    wl.setup(og, dev)
    line = measure(wl, args, og, dev, local, ws, 0.0 if args.no_cpu_baseline else args.cpu_budget)
    if ws > 1:
        torch.distributed.destroy_process_group()
    if line is None:
        return
    if args.workload == "pt" and not args.headline_only and args.ref_spp > 0:
        try:  # untimed: the frame's error against a long render, GPU and CPU
            line["image_stats"] = wl.image_stats(args.ref_spp)
        except Exception as e:
            line["image_stats"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if ws == 1 and args.workload == "pt" and not args.headline_only:
        # the other configurations, each in its own object of the same line
        del wl
        extras = {}
        for key, name in (("C0_ao", "ao"), ("C2_scivis", "scivis"), ("C3_batch", "batch")):
            t0 = time.perf_counter()
            try:
                w2 = WORKLOADS[name]()
                w2.setup(og, dev)
                sub = measure(w2, args, og, dev, local, 1, 0.0 if args.no_cpu_baseline else args.extra_cpu_budget)
                if name in ("ao", "scivis") and args.ref_spp > 0:
                    sub["image_stats"] = frame_relmse(w2, args.ref_spp)
                sub.pop("n_gpus", None)
                sub.pop("scaling", None)
                sub.pop("vs_baseline", None)
                sub.pop("data", None)
                if name == "batch":
                    # the same requests as one persistent launch per frame
                    try:
                        w2.set_mode("persistent")
                        p = measure(w2, args, og, dev, local, 1, 0.0)
                        sub["persistent"] = {k: p[k] for k in ("value", "ms_per_step", "e2e", "gpu_launches",
                                                               "latency", "clocks") if k in p}
                        sub["persistent"].update(mode="persistent", plan=p["config"]["plan"],
                                                 autotune=p["config"]["autotune"])
                    except Exception as e:
                        sub["persistent"] = {"error": "%s: %s" % (type(e).__name__, e)}
                del w2
            except Exception as e:  # a failed extra is reported, not fatal to the headline
                sub = {"error": "%s: %s" % (type(e).__name__, e)}
            sub["wall_s"] = round(time.perf_counter() - t0, 1)
            extras[key] = sub
        t0 = time.perf_counter()
        try:
            extras["C4_learned_cache"] = nrc_study(args, og, dev)
        except Exception as e:
            extras["C4_learned_cache"] = {"error": "%s: %s" % (type(e).__name__, e)}
        extras["C4_learned_cache"]["wall_s"] = round(time.perf_counter() - t0, 1)
        line["configs"] = extras
    print(json.dumps(line), flush=True)


def frame_relmse(wl, ref_spp):
    """relMSE of one frame of the workload (frame 0, its own spp) against a
    ref_spp-sample render of it on the GPU (untimed)."""
    og = wl.og
    spp = getattr(wl, "spp", 1)
    wl.reset()
    wl.step()
    ref = og.Frame(wl.fb.device, wl.w, wl.h, og.FB_COLOR | og.FB_ACCUM)
    frame = wl.fb
    wl.fb = ref
    try:
        for _ in range(max(1, ref_spp // spp)):
            wl.step()
    finally:
        wl.fb = frame
    out = {"reference_spp": int(max(1, ref_spp // spp) * spp), "frame_spp": spp,
           "relmse_gpu": _sig(og.relmse(frame, ref))}
    wl.reset()
    return out


def nrc_study(args, og, dev):
    """Learned-cache path tracer vs plain path tracer on the instanced-spheres
    scene: 1920x1080, 1 spp per frame, maxPathLength 8, static camera, up to
    `--nrc-frames` frames each; both compared by relMSE with a 4096-spp plain
    render (256 frames x 16 spp).  relMSE is taken over all pixels and over
    the pixels whose first hit is geometry (background pixels of constant
    radiance excluded).  Per arm: device seconds and frames to reach each
    relMSE level, end-to-end seconds (host-timed, including the relMSE
    reads), and a coarse curve."""
    from ospray_gb300 import scenes
    w, h = (int(x) for x in args.size.split("x")) if args.size else (1920, 1080)
    data = scenes.pt_instanced_scene(width=w, height=h)
    scene = og.Scene(dev)
    scenes.build_pt_scene(scene, data)
    scene.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                      else og.ambient_light(L["intensity"]) for L in data["lights"]])
    c = data["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    mats = og.materials_array(data["materials"])
    ref_frames = max(1, args.nrc_ref_spp // 16)
    t0 = time.perf_counter()
    ref = og.Frame(dev, w, h, og.FB_COLOR | og.FB_ACCUM | og.FB_DEPTH)
    p16 = og.pt_params(spp=16, max_path_length=8, roulette_path_length=3)
    for _ in range(ref_frames):
        og.render_pt(scene, cam, p16, mats, ref)
    dev.sync()
    ref_s = time.perf_counter() - t0
    p1 = og.pt_params(spp=1, max_path_length=8, roulette_path_length=3)
    b = scene.bounds()
    levels = (0.01, 0.005, 0.002, 0.001)

    def arm(render):
        fb = og.Frame(dev, w, h, og.FB_COLOR | og.FB_ACCUM)
        total = 0.0
        curve = []
        reached = {"all": {}, "hits": {}}
        e2e0 = time.perf_counter()
        with Clocks(0) as clk:
            for i in range(args.nrc_frames):
                e0 = dev.record_event()
                render(fb)
                e1 = dev.record_event()
                dev.sync()
                total += dev.event_ms(e0, e1) * 1e-3
                dev.release_event(e0)
                dev.release_event(e1)
                err = {"all": og.relmse(fb, ref), "hits": og.relmse_hits(fb, ref)[0]}
                for k, e in err.items():
                    for lv in levels:
                        if lv not in reached[k] and e <= lv:
                            reached[k][lv] = (i + 1, total, time.perf_counter() - e2e0)
                if (i + 1) in (1, 2, 4, 8, 16, 32, 64, 128, 256, 512) or i + 1 == args.nrc_frames:
                    curve.append({"frames": i + 1, "seconds": round(total, 4), "relmse": round(err["all"], 5),
                                  "relmse_hits": round(err["hits"], 5)})

        def table(k):
            return {str(lv): ({"frames": reached[k][lv][0], "device_s": round(reached[k][lv][1], 4),
                               "e2e_s": round(reached[k][lv][2], 4)} if lv in reached[k] else None) for lv in levels}
        return {"seconds_to_relmse_0.01": round(reached["all"][0.01][1], 4) if 0.01 in reached["all"] else None,
                "e2e_seconds_to_relmse_0.01": round(reached["all"][0.01][2], 4) if 0.01 in reached["all"] else None,
                "frames_to_relmse_0.01": reached["all"][0.01][0] if 0.01 in reached["all"] else None,
                "to_level": table("all"), "to_level_hit_pixels": table("hits"),
                "relmse_final": curve[-1]["relmse"], "relmse_hits_final": curve[-1]["relmse_hits"],
                "seconds_total": round(total, 4), "ms_per_frame": round(total / args.nrc_frames * 1e3, 3),
                "curve": curve, "clocks": clk.summary()}

    plain = arm(lambda fb: og.render_pt(scene, cam, p1, mats, fb))
    cache = og.RadianceCache(dev, b[:3], b[3:], learning_rate=1e-2, seed=1)
    # the cache's first frames train several epochs over their samples (it
    # starts from random parameters); every frame after them trains one
    learned = arm(lambda fb: og.render_pt_nrc(
        scene, cam, p1, mats, fb, cache,
        epochs=args.nrc_early_epochs if fb.frame_id < args.nrc_early_frames else 1))
    value = learned["seconds_to_relmse_0.01"]
    _, nhit = og.relmse_hits(ref, ref)

    def speedup(k, lv):
        a, bb = learned[k][str(lv)], plain[k][str(lv)]
        return round(bb["device_s"] / a["device_s"], 3) if a and bb else None
    return {"metric": "seconds to relMSE<=0.01 (learned cache)", "value": value, "unit": "s",
            "higher_is_better": False, "steps": args.nrc_frames, "dtype": "f32 render, bf16 MLP",
            "config": {"workload": "nrc_instanced_spheres_1080p", "width": w, "height": h, "spp_per_frame": 1,
                       "maxPathLength": 8, "roulettePathLength": 3, "frames": args.nrc_frames,
                       "hit_pixels": int(nhit),
                       "cache": "16-level hash grid (2^19 x 2 fp16 per level) + 64x4 ReLU MLP, bf16 tensor cores, "
                                "Adam 1e-2, 16384 training paths, 4 x 16384 samples per frame; the first %d frames "
                                "train %d epochs" % (args.nrc_early_frames, args.nrc_early_epochs),
                       "reference": {"spp": ref_frames * 16, "renderer": "plain GPU path tracer",
                                     "seconds": round(ref_s, 2)}},
            "learned": learned, "plain": plain,
            "speedup_time_to_relmse": {"all_pixels": {str(lv): speedup("to_level", lv) for lv in levels},
                                       "hit_pixels": {str(lv): speedup("to_level_hit_pixels", lv) for lv in levels}}}


def run_nrc(args):
    import torch  # noqa: F401  (device init order as the other arms)
    import ospray_gb300 as og
    dev = og.Device(0)
    line = nrc_study(args, og, dev)
    line.update({"n_gpus": 1, "warmup": 0, "scaling": "weak", "vs_baseline": None,
                 "data": "synthetic (seeded generators)"})
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="pt", choices=sorted(WORKLOADS) + ["nrc"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU-baseline work")
    ap.add_argument("--extra-cpu-budget", type=float, default=4.0,
                    help="seconds of CPU-baseline work for each of the other configurations")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--headline-only", action="store_true", help="skip the other configurations' objects")
    ap.add_argument("--batch-mode", default="graph", choices=["graph", "persistent"],
                    help="batch workload: wavefront kernels as a graph, or one persistent launch")
    ap.add_argument("--size", default=None, help="WxH override (profiling small cases; not the bench config)")
    ap.add_argument("--spp", type=int, default=None, help="spp override (path tracer; profiling only)")
    ap.add_argument("--scene", default=None,
                    help="path tracer scene override SEED,INSTANCES,LEVELS (the build tuner's held-out scene; "
                         "not the bench config)")
    ap.add_argument("--nrc-frames", type=int, default=256, help="frames per arm of the learned-cache study")
    ap.add_argument("--ref-spp", type=int, default=4096,
                    help="samples per pixel of the reference render for the headline frame's relMSE (0: skip)")
    ap.add_argument("--nrc-ref-spp", type=int, default=4096, help="spp of the learned-cache study's reference image")
    ap.add_argument("--nrc-early-frames", type=int, default=4, help="frames that train --nrc-early-epochs epochs")
    ap.add_argument("--nrc-early-epochs", type=int, default=4)
    args = ap.parse_args()
    if args.workload == "nrc":
        run_nrc(args)
        return
    if args.size or args.spp or args.scene:
        args.headline_only = True
        base = WORKLOADS[args.workload]
        w, h = (int(x) for x in args.size.split("x")) if args.size else (None, None)
        scene = [int(x) for x in args.scene.split(",")] if args.scene else None

        def make(base=base, w=w, h=h, spp=args.spp, scene=scene):
            kw = {}
            if w:
                kw.update(w=w, h=h)
            if spp and base is PTWorkload:
                kw.update(spp=spp)
            if scene and base is PTWorkload:
                kw.update(seed=scene[0], count=scene[1], levels=scene[2])
            wl = base(**kw)
            if scene:
                wl.config.update(scene_seed=scene[0])
            return wl
        WORKLOADS[args.workload] = make
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

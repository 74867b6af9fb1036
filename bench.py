#!/usr/bin/env python3
"""Benchmark of the batched multislice tilt series on GB300.

Workload (one "step"): the MsctKirkland tilt series on a synthetic specimen
-- 20000 atoms (C:N:O:S = 0.50:0.17:0.30:0.03, seeded) uniform in a
120^3 A cube centred in a 160 A box, 300 keV, 1024 x 1024 complex64 grid,
1 A slices (160 slice-steps per orientation), 180 rotations about y in 1
degree steps, two detector defoci (0 and 500 A), fp32 intensities.  The
metric is slice-steps/s = orientations x slices / wall time of the whole
step (host preparation, every pass, the free-space step and the intensity).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl ours (default) prints one JSON line with
  value        device-timed (CUDA events on the library's stream) with the
               specimen resident in host memory and images left in HBM
  e2e          the same call with host input and output buffers (pinned),
               host<->device copies inside the timed region
  roofline     the dominant kernel's algorithmic HBM bytes per launch over its
               event-timed duration, against MEASURED_PEAKS.json
  cpu_baseline the oracle's FP32 restatement of the reference on the host
               cores (a bounded sample of the same workload)
--impl reference times that CPU restatement alone (the reference's own code
cannot be built on the GPU host: its FFT library and XArrayLibrary are not
part of it).
Under torchrun every rank runs its own 180 orientations (weak scaling; the
orientations are independent, there is no collective on the data path).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tilt-series slice-steps/s (1024², FP32) batched vs per-angle GPU; err vs FP64"
UNIT = "slice-steps/s"
NX = 1024
FOV = 160.0
V0 = 300.0
DZ = 1.0
NANG = 180
DEFOCI = (0.0, 500.0)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler running during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index),
                                       "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def gpu_index(local_rank):
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    ids = [v for v in vis.split(",") if v.strip()]
    if ids and all(v.strip().isdigit() for v in ids):
        return int(ids[local_rank % len(ids)])
    return local_rank


def workload(rank, nang=NANG):
    from utr_public_gb300 import specimen
    spec = specimen.tilt_specimen(1002)
    angY = np.deg2rad(np.arange(nang, dtype=np.float64) * (NANG / nang))
    angZ = np.full(nang, 0.1 * rank)  # each rank its own orientations
    return spec, angZ, angY, np.array(DEFOCI)


def cpu_sample(threads, slices=(60, 70), spec=None):
    """The oracle's FP32 restatement of the reference on `threads` host
    threads, one orientation per thread (as MsctKirkland drives the
    reference), slices slices[0]+1..slices[1] of each orientation."""
    from oracle import oracle as orc
    O = orc.Oracle()
    if spec is None:
        spec, _, _, _ = workload(0)
    sp = orc.SeriesParams()
    sp.ax, sp.ctblengthz, sp.nx, sp.ny, sp.v0, sp.deltaz = FOV, FOV, NX, NX, V0, DZ
    sp.min_slice, sp.max_slices, sp.nmode = slices[0], slices[1], 0
    angY = np.deg2rad(np.linspace(0, 179, threads))
    angZ = np.zeros(threads)
    t0 = time.perf_counter()
    O.orientations_f32(sp, spec.Znum, spec.x, spec.y, spec.z, spec.occ, angZ, angY,
                       np.array([]), threads)
    dt = time.perf_counter() - t0
    steps = threads * (slices[1] - slices[0])
    return steps / dt, dt, steps


def oracle_slice_count():
    """Slices of the tilt-series workload (the reference's slice scan)."""
    from oracle import oracle as orc
    return int(orc.Oracle().slice_count(DZ, FOV))


# The other configurations, one subprocess each (fresh device state, own clock
# record): (workload, extra arguments, what the summary keeps of its error).
OTHER_CONFIGS = (
    ("C1_plain", ["--workload", "plain", "--steps", "20", "--warmup", "3"]),
    ("C3_phonon", ["--workload", "phonon", "--steps", "1", "--warmup", "3"]),
    ("C4_uneven", ["--workload", "uneven", "--steps", "1", "--warmup", "3", "--quick"]),
    ("C5_adjoint", ["--workload", "adjoint", "--steps", "3", "--warmup", "3", "--quick"]),
)


def run_other_configs(timeout_s=600):
    """One timed step (after three warm-ups) of every other configuration, each in
    its own process, summarised for the tilt line: value, e2e, dominant kernel's
    roofline fraction, clocks and the FP64 error of its own check."""
    out = {}
    for name, extra in OTHER_CONFIGS:
        t0 = time.perf_counter()
        try:
            r = subprocess.run([sys.executable, os.path.abspath(__file__), "--no-cpu-baseline",
                                "--no-per-angle"] + extra, capture_output=True, text=True,
                               timeout=timeout_s, cwd=ROOT)
            lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
            if r.returncode != 0 or not lines:
                out[name] = {"error": "exit %d: %s" % (r.returncode, r.stderr.strip()[-300:])}
                continue
            d = json.loads(lines[-1])
            roof = d.get("roofline") or {}
            e2e = d.get("e2e") or {}
            out[name] = {
                "metric": d.get("metric"), "value": d.get("value"), "unit": d.get("unit"),
                "ms_per_step": d.get("ms_per_step"), "steps": d.get("steps"),
                "warmup": d.get("warmup"), "workload": (d.get("config") or {}).get("workload"),
                "e2e": {"value": e2e.get("value"), "ms_per_step": e2e.get("ms_per_step")},
                "roofline": {"kernel": roof.get("kernel"), "frac": roof.get("frac"),
                             "achieved": roof.get("achieved"), "unit": roof.get("unit")},
                "gpu_launches": d.get("gpu_launches"), "clocks": d.get("clocks"),
                "err_vs_fp64": d.get("err_vs_fp64", d.get("err")),
                "wall_s": round(time.perf_counter() - t0, 1)}
        except Exception as ex:  # reported, not fatal
            out[name] = {"error": repr(ex)}
    return out


def host_memory_facts(ptr):
    """NUMA layout of the host and the node holding the page at `ptr` (a pinned
    host buffer): where the e2e copies land on a Grace host."""
    import ctypes
    nodes = sorted(n for n in os.listdir("/sys/devices/system/node") if n.startswith("node")) \
        if os.path.isdir("/sys/devices/system/node") else []
    facts = {"numa_nodes": len(nodes), "cpus": os.cpu_count()}
    try:
        bus = subprocess.run(["nvidia-smi", "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=20).stdout.split()[0]
        bus = bus.lower().replace("00000000:", "0000:")
        with open("/sys/bus/pci/devices/%s/numa_node" % bus) as f:
            facts["gpu_numa_node"] = int(f.read())
    except Exception:
        pass
    try:  # get_mempolicy(MPOL_F_NODE | MPOL_F_ADDR) on the buffer's first page
        libc = ctypes.CDLL("libc.so.6", use_errno=True)
        nr = {"aarch64": 236, "x86_64": 239}.get(os.uname().machine)
        mode = ctypes.c_int(-1)
        if nr and libc.syscall(nr, ctypes.byref(mode), None, ctypes.c_ulong(0),
                               ctypes.c_void_p(ptr), ctypes.c_ulong(3)) == 0:
            facts["pinned_buffer_numa_node"] = mode.value
    except Exception:
        pass
    return facts


def tilt_config(nang, nslices, world):
    """The `config` of the tilt-series line, shared by both arms."""
    return {"workload": "tilt series 1024^2, 160 A box, 20000 atoms in a 120^3 A cube, "
                        "300 keV, 1 A slices, 180 orientations (1 deg about y) x 2 "
                        "defoci (0, 500 A); seeded synthetic specimen",
            "orientations": nang,
            "slice_steps_per_step": nang * nslices * world, "images_per_step": nang * 2 * world,
            "l2": "inputs larger than L2 (wave and transmission buffers 2.9 GB per GPU)",
            "parallelism": "weak: one tilt series per GPU"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(threads, (60, 62))
    vals, total = [], 0.0
    for _ in range(args.steps):
        v, dt, _ = cpu_sample(threads, (60, 80))
        vals.append(v)
        total += dt
    v = float(np.median(vals))
    sample = ("%d orientations x slices 61-80 of the 180-orientation 1024^2 tilt series, one "
              "orientation per thread" % threads)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": dict(tilt_config(NANG, oracle_slice_count(), world), sample=sample),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def fp64_error_job(result):
    """Relative L2 error of one orientation (45 degrees) of the workload vs the
    FP64 oracle (run after the timed regions)."""
    try:
        from oracle import oracle as orc
        import utr_public_gb300 as msk
        spec, _, _, defoci = workload(0)
        O = orc.Oracle()
        sp = orc.SeriesParams()
        sp.ax, sp.ctblengthz, sp.nx, sp.ny, sp.v0, sp.deltaz = FOV, FOV, NX, NX, V0, DZ
        sp.max_slices, sp.min_slice = -1, 0
        t0 = time.perf_counter()
        ref_img, ref_ew, _ = O.orientation(sp, spec.Znum, spec.x, spec.y, spec.z, spec.occ,
                                           0.0, np.deg2rad(45.0), defoci, fp64=True,
                                           want_exit=True)
        result["oracle_s"] = time.perf_counter() - t0
        result["ref"] = (ref_img, ref_ew)
    except Exception as e:  # reported, not fatal
        result["error"] = repr(e)


ADJ_NX, ADJ_FOV, ADJ_V0, ADJ_NANG, ADJ_CHECKPOINT = 512, 64.0, 200.0, 90, 8
ADJ_METRIC = ("adjoint slice-steps/s (512², FP32, 64 slices x 90 orientations, forward + "
              "adjoint); dL/dv err vs FP64 adjoint and central differences")


def adjoint_check(result, v, S, target, angles, nvox, rp):
    """FP64 oracle adjoint and central differences (host threads) for a few
    orientations of the adjoint workload; v[a], target[a] host arrays."""
    try:
        from oracle import oracle as orc
        O = orc.Oracle()
        p = orc.StackParams()
        p.nx = p.ny = ADJ_NX
        p.ax = p.by = ADJ_FOV
        p.v0, p.deltaz, p.nslices = ADJ_V0, 1.0, S
        rng = np.random.default_rng(1005)
        threads = max(1, (os.cpu_count() or 2) - 1)
        out = []
        t0 = time.perf_counter()
        for a in angles:
            ta = time.perf_counter()
            g64, L64 = O.stack_adjoint(p, v[a], rp, target[a])
            result.setdefault("adjoint_s", []).append(time.perf_counter() - ta)
            vox = np.stack([rng.integers(0, S, nvox), rng.integers(0, ADJ_NX, nvox),
                            rng.integers(0, ADJ_NX, nvox)], axis=1)
            fd = O.stack_fd(p, v[a], rp, target[a], vox, nthreads=threads)
            out.append({"angle_index": int(a), "grad64": g64, "loss64": L64, "voxels": vox,
                        "fd": fd})
        result["cases"] = out
        result["seconds"] = time.perf_counter() - t0
        result["threads"] = threads
    except Exception as e:  # reported, not fatal
        result["error"] = repr(e)


def run_adjoint(args, rank, world, local_rank):
    """C5: per-orientation potential stacks of the plain specimen (splatted on
    the GPU), target images from the stacks perturbed by 1% Gaussian noise,
    L = sum (I - T)^2 at one detector plane, dL/dv with a checkpoint every 8
    slices (--adj-checkpoint K: every K).  One step = one msk_adjoint call over
    all 90 orientations.  `keep_all` times the same call with checkpoint 0, every
    wave and transmission of the forward pass kept in HBM (264 MiB per
    orientation, 24.9 GB) and nothing recomputed."""
    import torch
    import utr_public_gb300 as msk
    from utr_public_gb300 import specimen
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    msk.load()
    ctx = msk.Context(local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    spec = specimen.plain_specimen(1001)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    nang = args.adj_orientations
    angY = np.deg2rad(2.0 * np.arange(nang))
    angZ = np.full(nang, 0.1 * rank)
    s = msk.Series()
    s.nx = s.ny = ADJ_NX
    s.ctblength = s.ctblengthz = ADJ_FOV
    s.v0, s.deltaz = ADJ_V0, 1.0
    S = msk.slice_count(1.0, ADJ_FOV)
    v = torch.empty((nang, S, ADJ_NX, ADJ_NX), dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        ctx.potential_stack(s, *atoms, angZ, angY, v=v)
        gen = torch.Generator(device="cuda")
        gen.manual_seed(1005 + rank)
        vt = v * (1.0 + 0.01 * torch.randn(v.shape, generator=gen, device="cuda"))
    st = msk.Stack()
    st.nx = st.ny = ADJ_NX
    st.ax = st.by = ADJ_FOV
    st.v0, st.deltaz, st.nslices, st.checkpoint = ADJ_V0, 1.0, S, args.adj_checkpoint
    rp = np.array([0.0 - 0.5 * ADJ_FOV])  # detector defocus 0 from the box centre
    target = torch.empty((nang, 1, ADJ_NX, ADJ_NX), dtype=torch.float32, device="cuda")
    ctx.stack_images(st, vt, rp, images=target)
    grad = torch.empty_like(v)
    del vt
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()

    def timed(fn, k):
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1) / k
        if dist is not None:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    step = lambda: ctx.adjoint(st, v, rp, target, grad=grad)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(gpu_index(local_rank))
    ms = timed(step, args.steps)
    clk = clocks.stop()
    steps_per = nang * S
    value = world * steps_per / (ms / 1000.0)
    loss_dev, _ = ctx.adjoint(st, v, rp, target, grad=grad)
    # the orientations the oracle checks (0 and 44 degrees; --quick: 0 only)
    pick = [0] if args.quick else [0, nang // 4]
    g_dev = {a: grad[a].cpu().numpy() for a in pick}
    keep_all = None
    if args.adj_checkpoint != 0 and not args.quick:  # keeping every wave and transmission
        st.checkpoint = 0
        for _ in range(2):
            step()
        ms_keep = timed(step, args.steps)
        st.checkpoint = args.adj_checkpoint
        keep_all = {"value": world * steps_per / (ms_keep / 1000.0), "unit": UNIT,
                    "ms_per_step": ms_keep, "checkpoint": 0}
    # forward alone (images of the same stacks)
    fimg = torch.empty_like(target)
    ms_fwd = timed(lambda: ctx.stack_images(st, v, rp, images=fimg), 1 if args.quick else args.steps)
    # per-kernel attribution of one adjoint call
    ctx.profile(True)
    ms_serial = timed(step, 1)
    prof = ctx.profile_read()
    ctx.profile(False)
    # end to end: pinned host stacks, target and gradient
    hv = torch.empty(v.shape, dtype=torch.float32, pin_memory=True)
    hv.copy_(v)
    ht = torch.empty(target.shape, dtype=torch.float32, pin_memory=True)
    ht.copy_(target)
    hg = torch.empty(v.shape, dtype=torch.float32, pin_memory=True)
    k_e2e = max(1, min(args.steps, 2))
    ctx.adjoint(st, hv, rp, ht, grad=hg)
    ms_e2e = timed(lambda: ctx.adjoint(st, hv, rp, ht, grad=hg), k_e2e)
    ctx.profile(True)  # the copied bytes, from one more call (not the timed ones)
    ctx.adjoint(st, hv, rp, ht, grad=hg)
    prof_e2e = ctx.profile_read()
    ctx.profile(False)
    h2d = prof_e2e.get("copy_h2d", (0, 0.0, 0.0))[2]
    d2h = prof_e2e.get("copy_d2h", (0, 0.0, 0.0))[2]
    same = bool(torch.equal(hg, grad.cpu())) if rank == 0 else None
    kernels = {k: x for k, x in prof.items() if not k.startswith("copy_")}
    launches = int(sum(x[0] for x in kernels.values())) * args.steps
    dom = max(kernels, key=lambda k: kernels[k][1])
    n_l, t_ms, nbytes = kernels[dom]
    peak, peak_kind = peaks()
    achieved = (nbytes / n_l) / (t_ms / n_l / 1000.0) / 1e9
    if rank != 0:
        return
    err = None
    cpu = None
    if not args.no_fp64_check:
        check = {}
        adjoint_check(check, {a: v[a].cpu().numpy() for a in pick}, S,
                      {a: target[a].cpu().numpy() for a in pick}, pick, args.fd_voxels, rp)
        if "cases" in check:
            rl2 = lambda a, b: float(np.linalg.norm(np.asarray(a, np.float64) - b) /
                                     np.linalg.norm(b))
            cases = []
            for c in check["cases"]:
                g = g_dev[c["angle_index"]]
                ours = np.array([g[k, i, j] for k, i, j in c["voxels"]])
                cases.append({"orientation_deg": 2.0 * c["angle_index"],
                              "grad_rel_l2_vs_fp64_adjoint": rl2(g, c["grad64"]),
                              "grad_rel_l2_vs_central_fd": rl2(ours, c["fd"]),
                              "fd_voxels": int(len(ours))})
            err = {"cases": cases, "oracle_seconds": check["seconds"],
                   "oracle_threads": check["threads"]}
            t1 = min(check["adjoint_s"])
            cpu = {"value": S / t1, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": "the FP64 oracle's forward + adjoint of one orientation (%d slices, "
                             "512^2) on one host thread, %.1f s (the reference has no adjoint)"
                             % (S, t1)}
        else:
            err = {"error": check.get("error", "not run")}
    out = {
        "metric": ADJ_METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "adjoint: plain specimen (2000 atoms, 64 A box), 512^2, 64 "
                               "slices of 1 A, 200 keV, %d orientations (2 deg about y), " % nang +
                               "potentials splatted on the GPU, target from v(1 + 0.01 N(0,1)), "
                               "1 detector plane (defocus 0), " + (
                                   "every wave and transmission kept (checkpoint 0)"
                                   if args.adj_checkpoint == 0 else
                                   "checkpoint every %d slices" % args.adj_checkpoint),
                   "slice_steps_per_step": steps_per * world,
                   "l2": "inputs larger than L2 (stacks %.1f GB per GPU)"
                         % (nang * S * ADJ_NX * ADJ_NX * 4 / 1e9)},
        "keep_all": keep_all,
        "cpu_baseline": cpu,
        "forward_only": {"value": world * steps_per / (ms_fwd / 1000.0), "unit": UNIT,
                         "ms": ms_fwd, "adjoint_over_forward_time": ms / ms_fwd},
        "loss": loss_dev,
        "e2e": {"value": world * steps_per / (ms_e2e / 1000.0), "unit": UNIT,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": ms_e2e, "matches_device_output": same},
        "gpu_launches": launches * world,
        "ms_per_step_serialized": ms_serial,
        "kernels": {k: {"launches": x[0], "ms": round(x[1], 3),
                        "GBps": round(x[2] / (x[1] / 1000.0) / 1e9, 1) if x[1] > 0 else None}
                    for k, x in kernels.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind, "traffic": None,
                     "algorithmic_bytes_per_launch": nbytes / n_l},
        "clocks": clk,
        "err_vs_fp64": err,
    }
    print(json.dumps(out))


UTR_METRIC = ("UTR reconstruction voxels/s (1024^3 volume, CTF-3D, from the 180 x 1024^2 tilt "
              "series, FP32)")
UTR_UNIT = "voxels/s"


def utr_params(msk, n, xst):
    """UTR parameters of the reconstruction workload: an n^3 volume of voxel
    edge xst spanning the 160 A box, 300 keV, CTF-3D with the Ewald sphere
    correction, objective aperture 40 mrad, NSR 0.03, epsilon 1e-4 (the
    readme's example values), beta/delta 0.05."""
    u = msk.Utr()
    u.modality, u.f1, u.f2, u.nx, u.ny, u.xst = 0, 1.0, 0.0, n, n, xst
    u.zlo, u.zhi = -0.5 * n * xst, 0.5 * n * xst
    u.wl, u.aobj, u.ctf_mode, u.escc = 0.01968749, 40.0, 4, 1
    u.asigma, u.nsr, u.epsilon = 0.05, 0.03, 1e-4
    return u


def utr_cpu_sample(msk, imgs_small, ang, df, n, threads):
    """The oracle's FP64 restatement of UTR.cpp on the host cores: the whole
    reconstruction of an n^3 volume from the block-averaged images."""
    from oracle import oracle as orc
    O = orc.Oracle()
    u = utr_params(msk, n, FOV / n)
    p = orc.UtrParams()
    for name, _ in p._fields_:
        setattr(p, name, getattr(u, name))
    t0 = time.perf_counter()
    vol = O.utr_reconstruct(p, ang, df, imgs_small, nthreads=threads)
    return vol, time.perf_counter() - t0


def run_utr(args, rank, world, local_rank):
    """UTR reconstruction: the 180-orientation tilt series (defocus 500 A
    plane, simulated by this library's multislice, untimed) reconstructed
    into a 1024^3 volume.  One step = one msk_utr_reconstruct call."""
    import torch
    import utr_public_gb300 as msk
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    msk.load()
    ctx = msk.Context(local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    if args.profile_run:
        # for profilers: seeded smooth images, no multislice, a handful of calls
        n = args.utr_n
        g = torch.Generator(device="cuda")
        g.manual_seed(7)
        low = torch.randn((NANG, 1, n // 16, n // 16), generator=g, device="cuda")
        imgs = (1.0 + 0.05 * torch.nn.functional.interpolate(low, size=(n, n), mode="bilinear",
                                                             align_corners=False))[:, 0].contiguous()
        ang = np.stack([np.zeros(NANG), np.arange(NANG, dtype=np.float64)], axis=1)
        u = utr_params(msk, n, FOV / n)
        vol = torch.empty((ctx.utr_depth(u), n, n), dtype=torch.float32, device="cuda")
        for _ in range(2):
            ctx.utr_reconstruct(u, ang, np.full(NANG, 500.0), imgs, volume=vol)
        torch.cuda.synchronize()
        print(json.dumps({"profile_run": "utr", "n": n, "volume_abs_sum": float(vol.abs().sum())}))
        return
    spec, angZ, angY, _ = workload(rank, NANG)
    s = msk.Series()
    s.nx = s.ny = NX
    s.ctblength = s.ctblengthz = FOV
    s.v0, s.deltaz = V0, DZ
    timgs = torch.empty((NANG, 1, NX, NX), dtype=torch.float32, device="cuda")
    ctx.tilt_series(s, spec.Znum, spec.x, spec.y, spec.z, spec.occ, angZ, angY, [500.0],
                    images=timgs)
    torch.cuda.synchronize()
    # MsctKirkland's images are [nx][ny] (y fastest); UTR reads rows along y
    imgs = timgs[:, 0].transpose(1, 2).contiguous()
    del timgs
    n = args.utr_n
    if n != NX:  # a smaller volume: the images block-averaged to n^2
        f = NX // n
        imgs = imgs.reshape(NANG, n, f, n, f).mean(dim=(2, 4)).contiguous()
    ang = np.stack([np.rad2deg(angZ), np.rad2deg(angY)], axis=1)
    df = np.full(NANG, 500.0)
    u = utr_params(msk, n, FOV / n)
    nz = ctx.utr_depth(u)
    vol = torch.empty((nz, n, n), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()

    def timed(fn, k):
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1) / k
        if dist is not None:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    step = lambda: ctx.utr_reconstruct(u, ang, df, imgs, volume=vol)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(gpu_index(local_rank))
    ms = timed(step, args.steps)
    clk = clocks.stop()
    nvox = n * n * nz
    value = world * nvox / (ms / 1000.0)
    ctx.profile(True)
    ms_serial = timed(step, 1)
    prof = ctx.profile_read()
    ctx.profile(False)
    # end to end: pinned host images in, the host volume out
    himg = torch.empty(imgs.shape, dtype=torch.float32, pin_memory=True)
    himg.copy_(imgs)
    hvol = torch.empty(vol.shape, dtype=torch.float32, pin_memory=True)
    k_e2e = max(1, min(args.steps, 2))
    ctx.utr_reconstruct(u, ang, df, himg, volume=hvol)
    ms_e2e = timed(lambda: ctx.utr_reconstruct(u, ang, df, himg, volume=hvol), k_e2e)
    ctx.profile(True)  # the copied bytes, from one more call (not the timed ones)
    ctx.utr_reconstruct(u, ang, df, himg, volume=hvol)
    prof_e2e = ctx.profile_read()
    ctx.profile(False)
    h2d = prof_e2e.get("copy_h2d", (0, 0.0, 0.0))[2]
    d2h = prof_e2e.get("copy_d2h", (0, 0.0, 0.0))[2]
    # the gridding sums are float atomics: equal to the device run to rounding
    same = (float(torch.linalg.vector_norm(hvol - vol.cpu()) / torch.linalg.vector_norm(hvol))
            < 1e-6) if rank == 0 else None
    kernels = {k: x for k, x in prof.items() if not k.startswith("copy_")}
    launches = int(sum(x[0] for x in kernels.values())) * args.steps
    dom = max(kernels, key=lambda k: kernels[k][1])
    n_l, t_ms, nbytes = kernels[dom]
    peak, peak_kind = peaks()
    achieved = (nbytes / n_l) / (t_ms / n_l / 1000.0) / 1e9
    if rank != 0:
        return
    # FP64 oracle on a bounded sample: the same images block-averaged 4 x 4
    # to 256^2, a 256^3 volume; the GPU reconstructs the same sample
    cpu, err = None, None
    if not args.no_cpu_baseline and n % 4 == 0:
        small = imgs.reshape(NANG, n // 4, 4, n // 4, 4).mean(dim=(2, 4)).contiguous()
        small_np = small.cpu().numpy()
        threads = os.cpu_count() or 1
        m = n // 4
        ref, dt = utr_cpu_sample(msk, small_np, ang, df, m, threads)
        sample = ("180 images block-averaged to %d^2, a %d^3 volume (voxel %.4g A), the whole "
                  "reconstruction" % (m, m, FOV / m))
        cpu = {"value": m ** 3 / dt, "unit": UTR_UNIT, "cores": threads, "kind": "port",
               "sample": sample, "seconds": dt}
        us = utr_params(msk, m, FOV / m)
        got = ctx.utr_reconstruct(us, ang, df, small_np)
        err = {"volume_rel_l2_vs_fp64_%d" % m: float(np.linalg.norm(got - ref) /
                                                   np.linalg.norm(ref))}
    out = {
        "metric": UTR_METRIC, "value": value, "unit": UTR_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "UTR reconstruction: 180 orientations (1 deg about y) x %d^2 "
                               "images at defocus 500 A of the 20000-atom tilt specimen, %d^3 "
                               "volume of %.4g A voxels, CTF-3D + Ewald sphere correction, "
                               "aperture 40 mrad, NSR 0.03, epsilon 1e-4" % (n, n, FOV / n),
                   "voxels_per_step": nvox * world, "images_per_step": NANG * world,
                   "l2": "inputs larger than L2 (34 GB of gridding sums per GPU)"},
        "images_per_s": world * NANG / (ms / 1000.0),
        "e2e": {"value": world * nvox / (ms_e2e / 1000.0), "unit": UTR_UNIT,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": ms_e2e, "matches_device_output": same},
        "gpu_launches": launches * world,
        "ms_per_step_serialized": ms_serial,
        "kernels": {k: {"launches": x[0], "ms": round(x[1], 3),
                        "GBps": round(x[2] / (x[1] / 1000.0) / 1e9, 1) if x[1] > 0 else None}
                    for k, x in kernels.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind, "traffic": None,
                     "algorithmic_bytes_per_launch": nbytes / n_l},
        "clocks": clk,
        "cpu_baseline": cpu,
        "err_vs_fp64": err,
    }
    print(json.dumps(out))


UNEVEN_METRIC = ("uneven-batch slice-steps/s (64 specimens, 5e3-2e5 atoms, 256^2-2048^2, 1-90 "
                 "orientations, FP32, one CUDA graph)")


def run_uneven(args, rank, world, local_rank):
    """C4: 64 specimens of log-uniform atom count, field of view sqrt(2) x edge,
    grids drawn from {256, 512, 1024, 2048}, 1..90 orientations evenly over 180
    degrees, 300 keV, 1 A slices, two detector defoci; one msk_tilt_series_batch
    call (one CUDA graph) per step."""
    import torch
    import utr_public_gb300 as msk
    from utr_public_gb300 import specimen
    torch.cuda.set_device(local_rank)
    msk.load()
    ctx = msk.Context(local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    batch = specimen.uneven_batch(64, 1004)
    cases = []
    for sp_, n, nang in batch:
        aY = np.deg2rad(np.arange(nang) * (180.0 / nang))
        cases.append((sp_, n, np.full(nang, 0.1 * rank), aY))
    s = msk.Series()
    s.v0, s.deltaz = V0, DZ
    defoci = np.array(DEFOCI)
    imgs = [torch.empty((len(c[2]), len(defoci), c[1], c[1]), dtype=torch.float32, device="cuda")
            for c in cases]
    nsl = [msk.slice_count(DZ, c[0].fov) for c in cases]
    steps = [len(c[2]) * k for c, k in zip(cases, nsl)]

    def timed(fn, k):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    run = lambda graph, sel=None: ctx.tilt_series_batch(
        s, cases if sel is None else [cases[i] for i in sel], defoci, graph=graph,
        images=imgs if sel is None else [imgs[i] for i in sel])
    for _ in range(args.warmup):
        run(True)
    clocks = Clocks(gpu_index(local_rank))
    ms = timed(lambda: run(True), args.steps)
    clk = clocks.stop()
    total = sum(steps)
    value = world * total / (ms / 1000.0)
    ms_streams = None if args.quick else timed(lambda: run(False), 1)
    per_size = {}
    for n in (() if args.quick else (256, 512, 1024, 2048)):
        sel = [i for i, c in enumerate(cases) if c[1] == n]
        if not sel:
            continue
        run(True, sel)
        t = timed(lambda: run(True, sel), 1)
        st_ = sum(steps[i] for i in sel)
        per_size[str(n)] = {"specimens": len(sel), "slice_steps": st_, "ms": t,
                            "slice_steps_per_s": st_ / (t / 1000.0),
                            "column_plans": {p: msk.column_plan(local_rank, n, n, p)
                                             for p in ("band_limit", "propagate", "free_space")},
                            "row_plans": {"transmit": msk.row_plan(local_rank, n, n)}}
    ctx.profile(True)
    ms_serial = timed(lambda: run(False), 1)
    prof = ctx.profile_read()
    ctx.profile(False)
    kernels = {k: x for k, x in prof.items() if not k.startswith("copy_")}
    launches = int(sum(x[0] for x in kernels.values())) * args.steps
    # end to end: pinned host images
    host = [torch.empty(tuple(t.shape), dtype=torch.float32, pin_memory=True) for t in imgs]
    ctx.tilt_series_batch(s, cases, defoci, graph=True, images=host)  # warm: the host-image arena
    t0 = time.perf_counter()
    ctx.tilt_series_batch(s, cases, defoci, graph=True, images=host)
    ms_e2e = 1000.0 * (time.perf_counter() - t0)
    same = all(torch.equal(h, d.cpu()) for h, d in zip(host, imgs))
    dom = max(kernels, key=lambda k: kernels[k][1])
    n_l, t_ms, nbytes = kernels[dom]
    peak, peak_kind = peaks()
    achieved = (nbytes / n_l) / (t_ms / n_l / 1000.0) / 1e9
    if rank != 0:
        return
    err = None
    if not args.no_fp64_check:
        # FP64 oracle on one specimen per grid size (the one with the fewest atoms),
        # its first orientation; the four checks run on host threads
        try:
            import concurrent.futures as cf
            from oracle import oracle as orc
            O = orc.Oracle()

            def check(n):
                sel = [j for j in range(len(cases)) if cases[j][1] == n]
                i = min(sel, key=lambda j: cases[j][0].natom)
                sp_, _, aZ, aY = cases[i]
                p = orc.SeriesParams()
                p.ax, p.ctblengthz, p.nx, p.ny, p.v0, p.deltaz = sp_.fov, sp_.fov, n, n, V0, DZ
                p.max_slices, p.min_slice = -1, 0
                ref, _ = O.orientation(p, sp_.Znum, sp_.x, sp_.y, sp_.z, sp_.occ, aZ[0], aY[0],
                                       defoci, fp64=True)
                got = imgs[i][0].cpu().numpy()
                return {"specimen": i, "grid": n, "natom": sp_.natom,
                        "slices": msk.slice_count(DZ, sp_.fov),
                        "image_rel_l2": [float(np.linalg.norm(got[d] - ref[d]) /
                                               np.linalg.norm(ref[d])) for d in range(len(defoci))]}

            sizes = sorted({c[1] for c in cases})
            if args.quick:
                sizes = sizes[:1]
            with cf.ThreadPoolExecutor(len(sizes)) as ex:
                err = {"per_grid": list(ex.map(check, sizes))}
            err["max_image_rel_l2"] = max(max(e["image_rel_l2"]) for e in err["per_grid"])
        except Exception as ex:
            err = {"error": repr(ex)}
    out = {
        "metric": UNEVEN_METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "uneven batch: 64 specimens (seed 1004), natom log-uniform "
                               "5e3..2e5 at 0.1 atoms/A^3, FOV sqrt(2) x edge, grids "
                               "{256,512,1024,2048}^2, 1..90 orientations over 180 deg, 300 keV, "
                               "1 A slices, defoci 0 and 500 A",
                   "slice_steps_per_step": total, "images_per_step": 2 * sum(len(c[2]) for c in cases),
                   "l2": "inputs larger than L2 (tens of GB of waves)"},
        "per_size": per_size,
        "streams_without_graph": None if ms_streams is None else
                                 {"ms": ms_streams, "value": total / (ms_streams / 1000.0)},
        "e2e": {"value": total / (ms_e2e / 1000.0), "unit": UNIT, "h2d_bytes_per_step":
                int(prof.get("copy_h2d", (0, 0, 0))[2]),
                "d2h_bytes_per_step": int(sum(h.numel() * 4 for h in host)), "ms_per_step": ms_e2e,
                "matches_device_output": bool(same)},
        "gpu_launches": launches,
        "ms_per_step_serialized": ms_serial,
        "kernels": {k: {"launches": x[0], "ms": round(x[1], 3),
                        "GBps": round(x[2] / (x[1] / 1000.0) / 1e9, 1) if x[1] > 0 else None}
                    for k, x in kernels.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "traffic": None, "algorithmic_bytes_per_launch": nbytes / n_l},
        "clocks": clk,
        "err_vs_fp64": err,
    }
    print(json.dumps(out))


PLAIN_METRIC = "plain multislice slice-steps/s (256², FP32, one orientation); err vs FP32 reference and FP64"
PHONON_METRIC = ("frozen-phonon slice-steps/s (1024², FP32, 60 orientations x 32 configurations); "
                 "err vs FP64")


def _event_timer(torch, stream):
    def timed(fn, k):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k
    return timed


def _rl2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run_plain(args, rank, world, local_rank):
    """C1: the plain specimen (2000 atoms in [7, 57]^3, 64 A box), 256^2, 2 A slices,
    200 keV, one orientation, defocus 0: one msk_calculate call per step (host atoms,
    host exit wave) and the same orientation as a one-orientation msk_tilt_series
    (image left in HBM)."""
    import torch
    import utr_public_gb300 as msk
    from utr_public_gb300 import specimen
    torch.cuda.set_device(local_rank)
    msk.load()
    ctx = msk.Context(local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    timed = _event_timer(torch, stream)
    sp_ = specimen.plain_specimen(1001)
    atoms = (sp_.Znum, sp_.x, sp_.y, sp_.z, sp_.occ)
    param = msk.make_param(64.0, 64.0, 256, 256, 200.0, 2.0)
    nsl = msk.slice_count(2.0, 64.0)
    s = msk.Series()
    s.nx = s.ny = 256
    s.ctblength = s.ctblengthz = 64.0
    s.v0, s.deltaz = 200.0, 2.0
    img = torch.empty((1, 1, 256, 256), dtype=torch.float32, device="cuda")
    step = lambda: ctx.tilt_series(s, *atoms, [0.0], [0.0], [0.0], images=img)
    calc = lambda: ctx.calculate(param, *atoms, 64.0, 64.0)
    for _ in range(args.warmup):
        step()
        calc()
    clocks = Clocks(gpu_index(local_rank))
    ms = timed(step, max(args.steps, 20))
    clk = clocks.stop()
    t0 = time.perf_counter()
    k = max(args.steps, 20)
    for _ in range(k):
        pix = calc()
    ms_e2e = 1000.0 * (time.perf_counter() - t0) / k
    ctx.profile(True)
    step()
    prof = ctx.profile_read()
    ctx.profile(False)
    kernels = {kk: x for kk, x in prof.items() if not kk.startswith("copy_")}
    # the dominant kernel against the HBM copy peak (a 0.5 MB problem: the
    # launches are latency-bound, the fraction is low by nature)
    dom = max(kernels, key=lambda kk: kernels[kk][1])
    n_l, t_ms, nbytes = kernels[dom]
    peak, peak_kind = peaks()
    achieved = (nbytes / n_l) / (t_ms / n_l / 1000.0) / 1e9
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
            "traffic": None, "algorithmic_bytes_per_launch": nbytes / n_l}
    if rank != 0:
        return
    err = {}
    gold = os.path.join(ROOT, "tests", "golden", "ref_exit_c1_256.npz")
    if os.path.exists(gold):
        err["exit_wave_rel_l2_vs_reference_fp32"] = _rl2(pix, np.load(gold)["pix"])
    cpu = None
    if not args.no_fp64_check or not args.no_cpu_baseline:
        from oracle import oracle as orc
        O = orc.Oracle()
        if not args.no_fp64_check:
            ref64 = O.calculate(param, *atoms, 64.0, 64.0, fp64=True)
            err["exit_wave_rel_l2_vs_fp64"] = _rl2(pix, ref64)
            lam = O.wavelength(200.0)
            i64 = O.defocus(ref64, 64.0, 64.0, lam, 0.0 - 32.0, fp64=True)
            err["image_rel_l2_vs_fp64"] = _rl2(img[0, 0].cpu().numpy(), i64)
        if not args.no_cpu_baseline:
            t0 = time.perf_counter()
            n = 0
            while time.perf_counter() - t0 < 3.0:
                O.calculate(param, *atoms, 64.0, 64.0)
                n += 1
            dt = time.perf_counter() - t0
            cpu = {"value": n * nsl / dt, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": "%d calculate() calls of this workload on one host thread" % n}
    print(json.dumps({
        "metric": PLAIN_METRIC, "value": nsl / (ms / 1000.0), "unit": UNIT, "n_gpus": world,
        "steps": k, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "plain: 2000 atoms in [7,57]^3 A, 64 A box, 256^2, 2 A slices, "
                               "200 keV, one orientation, defocus 0 (seed 1001)",
                   "slice_steps_per_step": nsl,
                   "l2": "a 0.5 MB problem: L2-resident by nature (one exit wave)"},
        "e2e": {"value": nsl / (ms_e2e / 1000.0), "unit": UNIT,
                "h2d_bytes_per_step": int(prof.get("copy_h2d", (0, 0, 0))[2]),
                "d2h_bytes_per_step": 256 * 256 * 8, "ms_per_step": ms_e2e,
                "call": "msk_calculate, host atoms and exit wave"},
        "gpu_launches": int(sum(x[0] for x in kernels.values())) * k,
        "kernels": {kk: {"launches": x[0], "ms": round(x[1], 4)} for kk, x in kernels.items()},
        "roofline": roof,
        "clocks": clk, "cpu_baseline": cpu, "err": err}))


def run_phonon(args, rank, world, local_rank):
    """C3: the plain specimen in its 64 A box at 1024^2, 1 A slices, 200 keV, 60
    orientations in 3 degree steps, 32 thermal configurations (x, y, z += N(0,
    0.08^2), seeds (1003, c)), defocus 0, images averaged over configurations: one
    msk_tilt_series call per step."""
    import torch
    import utr_public_gb300 as msk
    from utr_public_gb300 import specimen
    torch.cuda.set_device(local_rank)
    msk.load()
    ctx = msk.Context(local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    timed = _event_timer(torch, stream)
    sp_ = specimen.plain_specimen(1001)
    atoms = (sp_.Znum, sp_.x, sp_.y, sp_.z, sp_.occ)
    nconf, nang = 32, 60
    disp = specimen.phonon_displacements(sp_, nconf, 0.08, 1003)
    angY = np.deg2rad(3.0 * np.arange(nang))
    angZ = np.full(nang, 0.1 * rank)
    s = msk.Series()
    s.nx = s.ny = 1024
    s.ctblength = s.ctblengthz = 64.0
    s.v0, s.deltaz = 200.0, 1.0
    nsl = msk.slice_count(1.0, 64.0)
    img = torch.empty((nang, 1, 1024, 1024), dtype=torch.float32, device="cuda")
    step = lambda: ctx.tilt_series(s, *atoms, angZ, angY, [0.0], nconfig=nconf,
                                   displacements=disp, images=img)
    for _ in range(args.warmup):
        step()
    clocks = Clocks(gpu_index(local_rank))
    ms = timed(step, args.steps)
    clk = clocks.stop()
    total = nang * nconf * nsl
    ctx.profile(True)
    ms_serial = timed(step, 1)
    prof = ctx.profile_read()
    ctx.profile(False)
    kernels = {kk: x for kk, x in prof.items() if not kk.startswith("copy_")}
    dom = max(kernels, key=lambda kk: kernels[kk][1])
    n_l, t_ms, nbytes = kernels[dom]
    peak, peak_kind = peaks()
    achieved = (nbytes / n_l) / (t_ms / n_l / 1000.0) / 1e9
    host = torch.empty((nang, 1, 1024, 1024), dtype=torch.float32, pin_memory=True)
    t0 = time.perf_counter()
    ctx.tilt_series(s, *atoms, angZ, angY, [0.0], nconfig=nconf, displacements=disp, images=host)
    ms_e2e = 1000.0 * (time.perf_counter() - t0)
    same = bool(torch.equal(host, img.cpu()))
    if rank != 0:
        return
    err = None
    if not args.no_fp64_check:
        # FP64 oracle: the average over the first two configurations of one orientation
        from oracle import oracle as orc
        O = orc.Oracle()
        p = orc.SeriesParams()
        p.ax, p.ctblengthz, p.nx, p.ny, p.v0, p.deltaz = 64.0, 64.0, 1024, 1024, 200.0, 1.0
        p.max_slices, p.min_slice = -1, 0
        a = nang // 3
        ref = sum(O.orientation(p, *atoms, angZ[a], angY[a], [0.0], fp64=True, disp=disp[c])[0][0]
                  for c in range(2)) / 2.0
        got, _ = ctx.tilt_series(s, *atoms, angZ[a:a + 1], angY[a:a + 1], [0.0], nconfig=2,
                                 displacements=disp[:2])
        err = {"orientation_deg": float(np.rad2deg(angY[a])), "configurations": 2,
               "image_rel_l2_vs_fp64": _rl2(got[0, 0], ref)}
    print(json.dumps({
        "metric": PHONON_METRIC, "value": world * total / (ms / 1000.0), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "frozen phonon: plain specimen (2000 atoms, 64 A box), 1024^2, "
                               "1 A slices, 200 keV, 60 orientations (3 deg about y) x 32 "
                               "configurations (rms 0.08 A, seeds (1003, c)), defocus 0, images "
                               "averaged over configurations",
                   "slice_steps_per_step": total * world, "images_per_step": nang,
                   "l2": "inputs larger than L2 (1920 waves, 46 GB of buffers)"},
        "e2e": {"value": world * total / (ms_e2e / 1000.0), "unit": UNIT,
                "h2d_bytes_per_step": int(prof.get("copy_h2d", (0, 0, 0))[2]),
                "d2h_bytes_per_step": int(host.numel() * 4), "ms_per_step": ms_e2e,
                "matches_device_output": same},
        "gpu_launches": int(sum(x[0] for x in kernels.values())) * args.steps,
        "ms_per_step_serialized": ms_serial,
        "kernels": {kk: {"launches": x[0], "ms": round(x[1], 3),
                         "GBps": round(x[2] / (x[1] / 1000.0) / 1e9, 1) if x[1] > 0 else None}
                    for kk, x in kernels.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "traffic": None, "algorithmic_bytes_per_launch": nbytes / n_l},
        "clocks": clk, "err_vs_fp64": err}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true")
    ap.add_argument("--no-per-angle", action="store_true")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="tilt workload: skip the one-step runs of the other configurations")
    ap.add_argument("--quick", action="store_true",
                    help="uneven / adjoint: the timed step, its profile, e2e and one FP64 "
                         "check only (the form the tilt line's other_configs runs)")
    ap.add_argument("--orientations", type=int, default=NANG,
                    help="orientations per step (180 for the headline workload)")
    ap.add_argument("--workload", default="tilt",
                    choices=["tilt", "adjoint", "uneven", "plain", "phonon", "utr"],
                    help="tilt: the 180-orientation 1024^2 tilt series (headline); plain: one "
                         "256^2 orientation; phonon: 60 orientations x 32 configurations at "
                         "1024^2; uneven: 64 specimens of uneven size in one graph; adjoint: "
                         "the 512^2 potential-stack adjoint over 90 orientations; utr: the UTR "
                         "reconstruction of the tilt series into a 1024^3 volume")
    ap.add_argument("--adj-checkpoint", type=int, default=ADJ_CHECKPOINT,
                    help="adjoint: slices per checkpoint (0: keep every wave and transmission "
                         "when memory allows)")
    ap.add_argument("--adj-orientations", type=int, default=ADJ_NANG,
                    help="adjoint: orientations per step (90 for the adjoint workload; fewer "
                         "keep a profiler capture within a few GB)")
    ap.add_argument("--fd-voxels", type=int, default=256,
                    help="central-difference voxels per checked orientation (adjoint)")
    ap.add_argument("--utr-n", type=int, default=NX,
                    help="volume edge of the utr workload (images block-averaged to it)")
    ap.add_argument("--profile-run", action="store_true",
                    help="one tilt series and its per-kernel table, for profilers")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.workload in ("plain", "phonon"):
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference",
                                  "metric": PLAIN_METRIC if args.workload == "plain" else PHONON_METRIC,
                                  "unavailable": "the reference arm is timed on the tilt series"}))
            return
        (run_plain if args.workload == "plain" else run_phonon)(args, rank, world, local_rank)
        return
    if args.workload == "uneven":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "metric": UNEVEN_METRIC,
                                  "unavailable": "timed for the tilt-series workload only"}))
            return
        run_uneven(args, rank, world, local_rank)
        return
    if args.workload == "utr":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "metric": UTR_METRIC,
                                  "unavailable": "UTR.exe needs XArrayLibrary, which the reference "
                                                 "does not include; the oracle port is timed as "
                                                 "cpu_baseline"}))
            return
        run_utr(args, rank, world, local_rank)
        return
    if args.workload == "adjoint":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "metric": ADJ_METRIC,
                                  "unavailable": "the reference has no adjoint"}))
            return
        run_adjoint(args, rank, world, local_rank)
        return

    if args.impl == "reference":
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
        run_reference(args, rank, world)
        return

    import torch
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    import utr_public_gb300 as msk
    msk.load()  # raises if the CUDA library is not built

    ctx = msk.Context(local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    nang = args.orientations
    spec, angZ, angY, defoci = workload(rank, nang)
    s = msk.Series()
    s.nx = s.ny = NX
    s.ctblength = s.ctblengthz = FOV
    s.v0, s.deltaz = V0, DZ
    nslices = msk.slice_count(DZ, FOV)
    steps_per = nang * nslices
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    images = torch.empty((nang, len(defoci), NX, NX), dtype=torch.float32, device="cuda")

    def step(img):
        ctx.tilt_series(s, *atoms, angZ, angY, defoci, images=img)

    def barrier():
        if dist is not None:
            dist.barrier()

    def timed(img, k):
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            step(img)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1) / k
        if dist is not None:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    if args.profile_run:
        ctx.profile(True)
        step(images)
        torch.cuda.synchronize()
        for k, v in sorted(ctx.profile_read().items(), key=lambda kv: -kv[1][1]):
            print("%-14s launches %6d  ms %9.3f  GB/s %8.1f" % (k, v[0], v[1],
                  v[2] / (v[1] / 1e3) / 1e9 if v[1] > 0 else 0.0))
        return

    for _ in range(args.warmup):
        step(images)
    torch.cuda.synchronize()

    # headline: the library's normal schedule (its two slice chains overlap)
    clocks = Clocks(gpu_index(local_rank))
    ms = timed(images, args.steps)
    clk = clocks.stop()
    value = world * steps_per / (ms / 1000.0)
    # per-kernel attribution: one more timed step with every launch bracketed by
    # CUDA events on its stream (the library then runs the passes in order)
    ctx.profile(True)
    ms_serial = timed(images, 1)
    prof = ctx.profile_read()
    ctx.profile(False)

    # end to end: host buffers (pinned), copies inside the timed region, the
    # library's normal schedule; the copied bytes from one more, profiled call
    # (profiling serialises the passes, so it is not the timed one)
    host_images = torch.empty((nang, len(defoci), NX, NX), dtype=torch.float32, pin_memory=True)
    step(host_images)
    ms_e2e = timed(host_images, max(1, min(args.steps, 3)))
    ctx.profile(True)
    step(host_images)
    torch.cuda.synchronize()
    prof_e2e = ctx.profile_read()
    ctx.profile(False)
    h2d = prof_e2e.get("copy_h2d", (0, 0.0, 0.0))[2]
    d2h = prof_e2e.get("copy_d2h", (0, 0.0, 0.0))[2]
    e2e_value = world * steps_per / (ms_e2e / 1000.0)
    # the image copies out (event-timed inside the library: each batch's images
    # on the library's third stream, beside the next batch's kernels; only the
    # last, small batch's copy follows the last kernel)
    cp = prof_e2e.get("copy_images_d2h", (0, 0.0, 0.0))
    copy_ms, copy_bytes = cp[1], cp[2]
    if rank == 0:
        same = torch.equal(host_images, images.cpu())
        host_facts = host_memory_facts(host_images.data_ptr())

    # the per-orientation comparison form (cuFFT, unfused kernels, one orientation
    # at a time) on a subset of the same orientations
    per_angle = None
    if not args.no_per_angle:
        sub = np.linspace(0, nang - 1, min(12, nang)).astype(int)
        pa_imgs = torch.empty((len(sub), len(defoci), NX, NX), dtype=torch.float32, device="cuda")
        try:
            ctx.tilt_series_per_angle(s, *atoms, angZ[sub[:1]], angY[sub[:1]], defoci,
                                      images=pa_imgs[:1])
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.tilt_series_per_angle(s, *atoms, angZ[sub], angY[sub], defoci, images=pa_imgs)
            e1.record(stream)
            torch.cuda.synchronize()
            pa_ms = e0.elapsed_time(e1)
            pa_val = len(sub) * nslices / (pa_ms / 1000.0)
            same = float(torch.linalg.norm(pa_imgs - images[sub]) / torch.linalg.norm(images[sub]))
            per_angle = {"value": pa_val, "unit": UNIT, "orientations_timed": int(len(sub)),
                         "ms": pa_ms, "batched_over_per_angle": value / pa_val,
                         "images_rel_l2_vs_batched": same}
            # this library's own fused passes, one orientation at a time (max_batch 1):
            # the batching's share of the gain, apart from the fusion's
            s1 = msk.Series()
            for f, _ in msk.Series._fields_:
                setattr(s1, f, getattr(s, f))
            s1.max_batch = 1
            ctx.tilt_series(s1, *atoms, angZ[sub[:1]], angY[sub[:1]], defoci, images=pa_imgs[:1])
            torch.cuda.synchronize()
            e0.record(stream)
            ctx.tilt_series(s1, *atoms, angZ[sub], angY[sub], defoci, images=pa_imgs)
            e1.record(stream)
            torch.cuda.synchronize()
            f_ms = e0.elapsed_time(e1)
            f_val = len(sub) * nslices / (f_ms / 1000.0)
            per_angle["fused_one_at_a_time"] = {"value": f_val, "ms": f_ms,
                                                "batched_over_it": value / f_val}
        except Exception as ex:  # reported, not fatal
            per_angle = {"error": repr(ex)}

    kernels = {k: v for k, v in prof.items() if not k.startswith("copy_")}
    launches = int(sum(v[0] for v in kernels.values())) * args.steps
    dom = max(kernels, key=lambda k: kernels[k][1])
    n_l, t_ms, nbytes = kernels[dom]
    peak, peak_kind = peaks()
    achieved = (nbytes / n_l) / (t_ms / n_l / 1000.0) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tf):
        d = json.load(open(tf)).get(dom)
        if d:
            traffic = (nbytes / n_l) * d["dram_bytes"] / d["algorithmic_bytes"]

    if rank != 0:
        return
    fp64 = {}
    if not args.no_fp64_check:
        fp64_error_job(fp64)
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, dt, n = cpu_sample(threads, (40, 160))  # ~10 s of CPU work on 16 cores
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d orientations x slices 41-160 (%d slice-steps, %.1f s) of this "
                         "workload, one orientation per thread" % (threads, n, dt)}
    err = None
    if not args.no_fp64_check:
        if "ref" in fp64:
            ref_img, ref_ew = fp64["ref"]
            sub = msk.Series()
            for f, _ in msk.Series._fields_:
                setattr(sub, f, getattr(s, f))
            img1, ew1, _ = ctx.tilt_series(sub, *atoms, [0.0], [np.deg2rad(45.0)], defoci,
                                           want_exit=True)
            rl2 = lambda a, b: float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))
            err = {"orientation_deg": 45.0, "exit_wave_rel_l2": rl2(ew1[0, 0], ref_ew),
                   "image_rel_l2": [rl2(img1[0, d], ref_img[d]) for d in range(len(defoci))],
                   "oracle_seconds": fp64.get("oracle_s")}
        else:
            err = {"error": fp64.get("error", "not run")}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": tilt_config(nang, nslices, world),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": ms_e2e,
                "matches_device_output": bool(same),
                "ms_over_device_step": ms_e2e - ms,
                "image_copy_ms_beside_kernels": copy_ms,
                "image_copy_GBps": copy_bytes / (copy_ms / 1000.0) / 1e9 if copy_ms > 0 else None,
                "host": host_facts},
        "gpu_launches": launches * world,
        "ms_per_step_serialized": ms_serial,
        "kernels": {k: {"launches": v[0], "ms": round(v[1], 3),
                        "GBps": round(v[2] / (v[1] / 1000.0) / 1e9, 1) if v[1] > 0 else None}
                    for k, v in kernels.items()},
        "per_angle_gpu": per_angle,
        # the column-pass schedules the tuner chose for this grid (FFT plan, tile)
        "column_plans": {p: msk.column_plan(local_rank, NX, NX, p)
                         for p in ("band_limit", "propagate", "free_space")},
        # and the transmit's (its row FFT plan)
        "row_plans": {"transmit": msk.row_plan(local_rank, NX, NX)},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": nbytes / n_l},
        "clocks": clk,
        "cpu_baseline": cpu,
        "err_vs_fp64": err,
    }
    if world == 1 and not args.no_other_configs:
        # the other configurations, after this line's own measurements
        out["other_configs"] = run_other_configs()
    print(json.dumps(out))


if __name__ == "__main__":
    main()

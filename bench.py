#!/usr/bin/env python
"""Benchmark of the GB300 IC path: IC particles/s at 1024^3 (ScalarI template,
20 modes, Box 1000 Mpc/h), fused FP32 form.

One "step" = one whole pass of the path (seed table -> white noise -> modal
non-Gaussian potential -> ZA + 2LPT -> particle positions and velocities) for
one realisation, with the Lagrangian positions and all fields resident in HBM.
Inputs are synthetic (BBKS transfer table, regular particle lattice,
coefficient table from the reference Decomposer); the working set (~130 GB)
is far above L2, so no flush is needed between steps.

  python bench.py [--gpus N --steps K --warmup W]           (GPU arm)
  python bench.py --impl reference [...]                    (CPU reference arm)

Under torchrun (N > 1) every rank runs its own realisation (replicas: the
path has no exchange step), timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

TABLES = os.path.join(ROOT, "tests", "golden", "tables")
METRIC = "IC particles/s at 1024^3 (fused FP32 form)"
UNIT = "particles/s"

WORKLOADS = {
    # name: (Nmesh, Box, table, N_modes, Nmax, Fnl)
    "scalarI_m20_n1024": (1024, 1000.0, "scalarI_m20_L1000_n1024", 20, 1024, 100.0),
    "scalarI_m12_n512": (512, 1000.0, "scalarI_m12_L1000_n512", 12, 512, 100.0),
    # the 1024^3 workload's 20-mode table on a 512^3 grid (per-launch DRAM
    # traffic of this case times 8 is the 1024^3 traffic: same term list)
    "scalarI_m20_n512": (512, 1000.0, "scalarI_m20_L1000_n1024", 20, 1024, 100.0),
    "scalarI_m12_n256": (256, 1000.0, "scalarI_m12_L1000_n512", 12, 512, 100.0),
    "local_m8_n128": (128, 500.0, "local_m8_L500_n128", 8, 128, 10.0),
    # the large single run: 1536^3, Box 2000, resonant template (LogResonance
    # w = 10, 20 modes); the slab form (fused fields would need 308 GB)
    "logres_m20_n1536": (1536, 2000.0, "logres_w10_m20_L2000_n1536", 20, 1536, 100.0),
}
# workloads the fused form's fields do not fit: the slab form, this many x-slabs
SLAB_DEFAULT = {"logres_m20_n1536": 8}
# Batching: 32 realisations at 256^3, Box 500, each with its own seed and a
# template cycling over Local / Equilateral / ScalarI (mass 0.5, 1, 1.5, 1.75)
# with 6..20 modes, run as one CUDA graph (aar_batch_*).
BATCH_TEMPLATES = [("local_m6_L500_n256", 6, 10.0), ("equil_m9_L500_n256", 9, 100.0),
                   ("scalarI_m10_L500_n256", 10, 100.0), ("scalarI_m13_L500_n256_mu0p5", 13, 100.0),
                   ("scalarI_m16_L500_n256_mu1p5", 16, 100.0), ("scalarI_m20_L500_n256_mu1p75", 20, 100.0)]
BATCH_WORKLOADS = {"batch32_n256": (32, 256, 500.0)}
# modal decompositions (Decomposer.go): model, N_modes, Lbox, Nmax, model keywords, reference table
DECOMP_WORKLOADS = {
    "decomp_logres_m20": ("LogResonance", 20, 2000.0, 1536, {"w_res": 10.0, "phi": 0.0}, "logres_w10_m20_L2000_n1536"),
    "decomp_local_m20": ("Local", 20, 1000.0, 1024, {}, None),
}
# the covariance build alone (aar_tetra_covariance): N_modes, Lbox, Nmax, k_grid_size of the basis
COV_WORKLOADS = {"cov_m20_L2000_n1536": (20, 2000.0, 1536, 150), "cov_m12_L1000_n512_k96": (12, 1000.0, 512, 96)}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", default="scalarI_m20_n1024",
                    choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS) + sorted(DECOMP_WORKLOADS) + sorted(COV_WORKLOADS))
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default schedule (no aar_autotune)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-n", type=int, default=128)
    ap.add_argument("--split-modal", action="store_true",
                    help="under torchrun: all ranks make one realisation together, the modal sum split over r "
                         "(aarambam_gb300.modal_split; one reduce to rank 0, which runs 2LPT and the read-out)")
    ap.add_argument("--stages-only", action="store_true",
                    help="profiling case: the field stages (noise, modal, 2LPT) only, no particle arrays")
    ap.add_argument("--rows-harness", type=int, default=0, metavar="NROWS",
                    help="profiling case: the modal row kernel alone on NROWS rows (aar_profile_modal_rows)")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 cuFFT forms (reference loop structure and regrouped, 1 step each)")
    ap.add_argument("--slab", type=int, default=0, metavar="S",
                    help="run the slab form (AAR_SLAB_FP32) with S x-slabs (default for workloads whose fused "
                         "fields do not fit one GPU)")
    ap.add_argument("--slab-device-out", action="store_true",
                    help="slab form: particles into device buffers instead of pinned host memory")
    return ap.parse_args()


def make_cfg(wl: str, seed: int) -> dict:
    N, box, tab, M, nmax, fnl = WORKLOADS[wl]
    return dict(Nmesh=N, Nsample=N, Nmax=nmax, Box=box, Seed=seed, Fnl=fnl, N_modes=M, table=tab, Omega=0.3,
                OmegaLambda=0.7, HubbleParam=0.7, Sigma8=0.8, PrimordialIndex=0.965, Redshift=49.0,
                FixedAmplitude=0, PhaseFlip=0, SphereMode=0, UnitLength_in_cm=3.085678e24, UnitMass_in_g=1.989e43,
                UnitVelocity_in_cm_per_s=1e5, InputSpectrum_UnitLength_in_cm=3.085678e24)


def load_tables(tab: str, M: int):
    from aarambam_gb300 import tables
    d = os.path.join(TABLES, tab)
    alpha = tables.load_alpha(os.path.join(d, "AlphaTable.dat"), M)
    x0 = tables.load_x0(os.path.join(d, "AiTable.dat"), M)
    k, t = tables.bbks_transfer()
    return alpha, x0, k, t


def active_r(alpha: np.ndarray) -> int:
    M = alpha.shape[0]
    rs = {r for p in range(M) for q in range(p, M) for r in range(q, M) if alpha[p, q, r] != 0}
    if M > 2 and alpha[0, 1, 2] != 0:
        rs |= {1, 2}
    return len(rs)


def active_pairs(alpha: np.ndarray) -> int:
    """(N_i, N_j) pairs whose FFTs the reference does not skip (main.c:747-759)."""
    M = alpha.shape[0]
    return sum(1 for p in range(M) for q in range(p, M) if any(alpha[p, q, r] != 0 for r in range(q, M)))


def lattice_positions(N: int, box: float, device):
    """Lagrangian positions of an N^3 lattice in the reference's particle
    order (read_glass.c:181-214 with a 64^3 lattice glass tiled N/64 times
    when N >= 64), float32 [N^3, 3] on the device."""
    import torch
    g = min(N, 64)
    tile = N // g
    glass = (torch.arange(g, dtype=torch.float64) * (100.0 / g)).float().double()
    bt = box / tile
    n = torch.arange(N, device=device)
    # index of a particle: ((ti*tile + tj)*tile + tk) * g^3 + (gi*g + gj)*g + gk
    ti, gi = n // g, n % g
    coord = (glass.to(device)[gi] / 100.0 * bt + ti.double() * bt).float()  # per-axis value of lattice index
    # assemble in particle order
    idx = torch.arange(N ** 3, device=device, dtype=torch.int64)
    gl, t = idx % (g ** 3), idx // (g ** 3)
    gx, gy, gz = gl // (g * g), (gl // g) % g, gl % g
    tx, ty, tz = t // (tile * tile), (t // tile) % tile, t % tile
    pos = torch.stack([coord[tx * g + gx], coord[ty * g + gy], coord[tz * g + gz]], dim=1).contiguous()
    return pos


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def alg_bytes(name: str, N: int, M: int, R: int, npart: int) -> float:
    """Algorithmic HBM bytes of one launch of each kernel: every field it must
    read and write once (complex half spectrum, F = 8 N^2 (N/2+1) bytes)."""
    F = 8.0 * N * N * (N // 2 + 1)
    table = {
        "seedtable": 4.0 * N * N, "noise": F + 4.0 * N * N,
        "modal_xinv": (1 + M) * F, "modal_ypass_inv": 2 * M * F, "modal_rows": (M + R) * F,
        "modal_ypass_fwd": 2 * R * F, "modal_xfwd": 2 * R * F, "modal_acc": (R + 2) * F,
        # 2LPT: x passes write one field per distinct x factor (Hessians 3,
        # displacements 2 + 2) and the y passes fan them out to 6
        "lpt_scale_twb": 2 * F, "lpt_xinv_hess": 4 * F, "lpt_ypass_inv_hess": 9 * F, "lpt_rows_source": 7 * F,
        "lpt_ypass_fwd_source": 2 * F, "lpt_xfwd_source": 2 * F, "lpt_xpsi2": 3 * F, "lpt_xpsi1": 3 * F,
        "lpt_ypass_inv_disp": 10 * F,
        "lpt_rows_c2r": 12 * F, "readout": 6 * 4.0 * N ** 3 + 36.0 * npart,
        # displacement rows with the lattice read-out fused: 6 fields in, Pos / Vel out
        "lpt_rows_readout": 6 * F + 24.0 * npart,
    }
    return table.get(name, float("nan"))


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d.get("bf16_tflops", 1900.0)),
                "source": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def traffic_for(kernel: str, N: int):
    """dram bytes per launch from a committed ncu summary, scaled to N."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
        e = d[kernel]
        return e["bytes_per_launch"] * (N / e["N"]) ** 3
    except (OSError, KeyError, ValueError):
        return None


def cpu_baseline(wl: str, n_sample: int, steps: int = 1) -> dict:
    """The FP64 oracle (the reference algorithm restated in C, OpenMP over all
    host cores) on a bounded sample of the workload: the same coefficient
    table and path at n_sample^3."""
    from oracle import oracle as O
    O.build()
    cfg = make_cfg(wl, 1234)
    cfg.update(Nmesh=n_sample, Nsample=n_sample)
    alpha, x0, k, t = load_tables(cfg["table"], cfg["N_modes"])
    o = O.Oracle(cfg, k, t)
    g = np.arange(n_sample, dtype=np.float64) * (cfg["Box"] / n_sample)
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    lagr = np.stack([x.ravel(), y.ravel(), z.ravel()], 1).astype(np.float32)
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        ref = o.run(alpha, x0, lagr)
        ts.append(time.perf_counter() - t0)
    sec = min(ts)
    cores = os.cpu_count()
    out = {"value": n_sample ** 3 / sec, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"oracle FP64 C restatement of the reference path (same {cfg['N_modes']}-mode table, "
                     f"reference loop structure, OpenMP) on {n_sample}^3 particles/grid, {sec:.2f} s/step, "
                     f"{os.uname().machine}"}
    return out, (cfg, alpha, x0, k, t, lagr, ref)


def _rel(a, b) -> float:
    a, b = np.asarray(a), np.asarray(b)
    dt = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    a, b = a.astype(dt), b.astype(dt)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _delta(psi1: np.ndarray, box: float) -> np.ndarray:
    """delta = -div psi1 on the grid (spectral derivative), [3, N, N, N] in."""
    N = psi1.shape[1]
    k = 2 * np.pi / box * np.fft.fftfreq(N, 1.0 / N)
    kz = 2 * np.pi / box * np.arange(N // 2 + 1)
    ks = [k[:, None, None], k[None, :, None], kz[None, None, :]]
    d = sum(1j * ks[a] * np.fft.rfftn(psi1[a]) for a in range(3))
    return -np.fft.irfftn(d, s=(N, N, N), axes=(0, 1, 2))


def precision_report(sample) -> dict:
    """Relative RMS errors of the fused FP32 form (and of the plain FP64 form's
    displacements) against the FP64 oracle on the cpu_baseline sample."""
    import torch
    from aarambam_gb300.ic import ICGenerator
    cfg, alpha, x0, k, t, lagr, ref = sample
    N, box = cfg["Nmesh"], cfg["Box"]
    dev = torch.device("cuda", torch.cuda.current_device())
    gl = torch.from_numpy(lagr).to(dev)
    g = ICGenerator(cfg, alpha, x0, k, t)
    g.stage("noise")
    g.stage("modal")
    phik = g.spectrum().cpu().numpy()
    g.stage("lpt")
    f = np.stack([g.field(i).double().cpu().numpy() for i in range(6)])
    pos, _ = g.readout(gl)
    o_tot = ref["total"][..., 0] + 1j * ref["total"][..., 1]
    o_disp = ref["disp"]

    def dspl(p):
        d = np.asarray(p, np.float64) - lagr.astype(np.float64)
        return d - box * np.round(d / box)
    want = dspl(ref["pos"].reshape(-1, 3))
    out = {"n": N, "phi": _rel(phik, o_tot), "delta": _rel(_delta(f[:3], box), _delta(o_disp[:3], box)),
           "psi1": _rel(f[:3], o_disp[:3]), "psi2": _rel(f[3:], o_disp[3:]),
           "displacement": _rel(dspl(pos.cpu().numpy()), want)}
    del g
    gp = ICGenerator(cfg, alpha, x0, k, t, precision="fp64")
    pp, _ = gp.run(gl)
    out["plain_fp64_displacement"] = _rel(dspl(pp.cpu().numpy()), want)
    del gp
    torch.cuda.empty_cache()
    return {k_: (round(v, 12) if isinstance(v, float) else v) for k_, v in out.items()}


def precision_vs_plain(wl: str = "scalarI_m12_n512") -> dict:
    """Relative RMS particle-displacement difference of the fused FP32 form
    against the plain FP64 GPU form at full size (the 512^3 / 12-mode
    workload; the FP64 oracle is too slow there)."""
    import torch
    from aarambam_gb300.ic import ICGenerator
    cfg = make_cfg(wl, 1234)
    N, box = cfg["Nmesh"], cfg["Box"]
    alpha, x0, k, t = load_tables(cfg["table"], cfg["N_modes"])
    dev = torch.device("cuda", torch.cuda.current_device())
    lagr = lattice_positions(N, box, dev)
    g = ICGenerator(cfg, alpha, x0, k, t)
    pf, _ = g.run(lagr)
    del g
    torch.cuda.empty_cache()
    gp = ICGenerator(cfg, alpha, x0, k, t, precision="fp64")
    pp, _ = gp.run(lagr)
    del gp
    torch.cuda.empty_cache()

    def dspl(p):
        d = p.double() - lagr.double()
        return d - box * torch.round(d / box)
    want = dspl(pp)
    err = float(torch.linalg.vector_norm(dspl(pf) - want) / torch.linalg.vector_norm(want))
    return {"workload": wl, "n": N, "displacement": round(err, 12)}


def replica_seed(rank: int) -> int:
    """Replicas run independent realisations: the seed of rank r is 1234 + r."""
    return 1234 + rank


def max_over_ranks(seconds: float, device=None) -> float:
    """The slowest rank's time (the job ends when it does); the process
    group's backend does the reduction (NCCL on GPUs, gloo in the CPU test)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return seconds
    tt = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_rate(world: int, steps: int, units_per_step: int, seconds: float) -> float:
    """Whole-job throughput: units of all ranks over the slowest rank's time."""
    return world * steps * units_per_step / seconds


def gpu_arm(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from aarambam_gb300 import _lib
    from aarambam_gb300.ic import ICGenerator
    _lib.load(build_if_missing=True)

    cfg = make_cfg(args.workload, replica_seed(rank))
    N, M = cfg["Nmesh"], cfg["N_modes"]
    alpha, x0, k, t = load_tables(cfg["table"], M)
    R = active_r(alpha)
    gen = ICGenerator(cfg, alpha, x0, k, t)
    # the plan's schedule, chosen by timing the candidates on this GPU
    tuned = [] if args.no_autotune else [l for l in gen.autotune().splitlines() if l.strip()]
    # particles: the reference's default glass, a regular 64^3 lattice, tiled
    # N/64 times (read_glass.c:129-214) -- aar_run_lattice, no glass array
    gn = min(N, 64)
    tile = N // gn
    npart = N ** 3
    pos = torch.empty((npart, 3), dtype=torch.float32, device=dev)
    vel = torch.empty_like(pos)

    def step():
        gen.run_lattice(gn, 100.0, tile, pos, vel)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    clk = Clocks(local)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        step()
        launches += gen.launches
    e1.record(stream)
    barrier()
    clocks = clk.stop()
    elapsed = max_over_ranks(e0.elapsed_time(e1) / 1e3, dev)
    value = job_rate(world, args.steps, npart, elapsed)

    # the same realisations from an N^3 array of Lagrangian positions in HBM
    # (aar_run: the general trilinear read-out), for comparison
    lagr = lattice_positions(N, cfg["Box"], dev)
    gen.run(lagr, pos, vel)
    barrier()
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ka = max(1, min(args.steps, 3))
    a0.record(stream)
    for _ in range(ka):
        gen.run(lagr, pos, vel)
    a1.record(stream)
    barrier()
    value_array = job_rate(world, ka, npart, max_over_ranks(a0.elapsed_time(a1) / 1e3, dev))

    # per-kernel times of one profiled step (events on the launching stream)
    buf = __import__("ctypes").create_string_buffer(1 << 16)
    gen.L.aar_profile_enable(gen.h, 1)
    for _ in range(max(1, min(args.steps, 2))):
        step()
    gen.L.aar_profile_report(gen.h, buf, len(buf))
    gen.L.aar_profile_enable(gen.h, 0)
    kernels = {}
    for line in buf.value.decode().strip().splitlines():
        nm, cnt, ms = line.split(",")
        kernels[nm] = {"launches": int(cnt), "ms": float(ms)}
    tot = sum(v["ms"] for v in kernels.values())
    pk = peaks()
    dom = max(kernels, key=lambda n: kernels[n]["ms"])
    for nm, v in kernels.items():
        per = v["ms"] / v["launches"] / 1e3
        v["share"] = round(v["ms"] / tot, 4)
        v["gbs"] = round(alg_bytes(nm, N, M, R, npart) / per / 1e9, 1)
    d_per = kernels[dom]["ms"] / kernels[dom]["launches"] / 1e3
    achieved = alg_bytes(dom, N, M, R, npart) / d_per / 1e9
    roofline = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4),
                "traffic": traffic_for(dom, N), "peak_source": pk["source"]}
    # whole path against the algorithmic byte count 4 N^3 (46 + 9 M)
    b_path = 4.0 * N ** 3 * (46 + 9 * M)
    path_roof = {"bytes_per_step": b_path, "achieved": round(b_path / (elapsed / args.steps) / 1e9, 1),
                 "frac": round(b_path / (elapsed / args.steps) / 1e9 / pk["hbm_gbs"], 4)}

    e2e = None
    if not args.no_e2e:
        # end to end on the reference's dataflow (read_glass.c:129-214): the
        # 64^3 lattice glass goes in (host), positions and velocities come
        # back into pinned host buffers.  aar_run_glass_host_async: each
        # step's copy-out overlaps the next step's fields; the timed region
        # ends when every copy is on the host.
        g = min(N, 64)
        tile = N // g
        from aarambam_gb300.gadget import lattice_glass
        glass = torch.from_numpy(lattice_glass(g, 100.0)).pin_memory().numpy()
        h_pos = torch.empty((npart, 3), dtype=torch.float32, pin_memory=True)
        h_vel = torch.empty((npart, 3), dtype=torch.float32, pin_memory=True)
        out = (h_pos, h_vel, None)
        gen.run_glass_host(glass, 100.0, tile, out=out)  # staging allocation, warm-up
        barrier()
        # a finite run ends with one copy-out that nothing overlaps: at 10 or
        # more realisations that tail is a tenth of one or less (the
        # pipeline's steady state is max(fields, copy-out) per realisation)
        ks = max(10, min(args.steps, 20))
        t0 = time.perf_counter()
        for _ in range(ks):
            gen.run_glass_host(glass, 100.0, tile, out=out, wait=False)
        gen.wait_host_copies()
        barrier()
        te = max_over_ranks(time.perf_counter() - t0, dev)
        # the synchronous entry point (each call returns with its particles on the host)
        t1 = time.perf_counter()
        for _ in range(2):
            gen.run_glass_host(glass, 100.0, tile, out=out)
        barrier()
        ts = max_over_ranks(time.perf_counter() - t1, dev) / 2
        # same particles as the device-resident run (the same tiled lattice glass)
        step()
        barrier()
        same = bool(torch.equal(h_pos, pos.cpu()) and torch.equal(h_vel, vel.cpu()))
        # copy bandwidth from the device to the pinned host buffers
        c0, c1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
        c0.record(stream)
        h_pos.copy_(pos, non_blocking=True)
        h_vel.copy_(vel, non_blocking=True)
        c1.record(stream)
        torch.cuda.synchronize()
        d2h_gbs = 24 * npart / (c0.elapsed_time(c1) / 1e3) / 1e9
        e2e = {"value": job_rate(world, ks, npart, te), "unit": UNIT, "h2d_bytes_per_step": 12 * g ** 3,
               "d2h_bytes_per_step": 24 * npart, "steps": ks, "d2h_gbs": round(d2h_gbs, 1),
               "sync_value": job_rate(world, 1, npart, ts), "matches_device_run": same,
               "api": "aar_run_glass_host_async (C ABI: host glass in, host Pos/Vel out, pinned; copy-out on side "
                      "streams overlapping the next realisation)"}
        del h_pos, h_vel

    plain = {}
    if not args.no_plain:
        # plain FP64 cuFFT forms, one step each after their set-up: the
        # reference loop structure (M + 2P + 41 transforms) and the regrouped
        # modal sum (at most 2M + 13), which separates the algorithmic gain
        # of the regrouping from the FP32 / fusion gain
        del gen
        torch.cuda.empty_cache()
        P = active_pairs(alpha)
        for key, form, nfft in (("plain_fp64", "fp64", M + 2 * P + 41),
                                ("plain_fp64_regrouped", "fp64_regrouped", M + R + 13)):
            gp = ICGenerator(cfg, alpha, x0, k, t, precision=form)
            gp.prepare()
            barrier()
            p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            p0.record(stream)
            gp.run(lagr, pos, vel)
            p1.record(stream)
            barrier()
            tp = p0.elapsed_time(p1) / 1e3
            plain[key] = {"value": npart / tp, "unit": UNIT, "ms_per_step": 1e3 * tp, "steps": 1,
                          "fused_speedup": round(tp / (elapsed / args.steps), 2), "transforms": nfft,
                          "form": "cuFFT Z2D/D2Z FP64 + separate pointwise kernels, "
                                  + ("reference loop structure" if form == "fp64" else "regrouped modal sum")}
            del gp
            torch.cuda.empty_cache()

    cpu = None
    precision = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, sample = cpu_baseline(args.workload, args.cpu_sample_n)
        precision = precision_report(sample)
        precision["fused_vs_plain_fp64_at_512"] = precision_vs_plain()

    if rank == 0:
        out = {"metric": METRIC, "value": value, "value_lagrangian_array": value_array, "unit": UNIT,
               "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {"workload": f"{args.workload}: Nmesh={N}^3 particles, Box={cfg['Box']} Mpc/h, "
                                      f"{cfg['table']} ({M} modes, {R} active r), Fnl={cfg['Fnl']}, BBKS T(k), "
                                      f"z=49, particles from a {gn}^3 lattice glass tiled {tile}^3 times "
                                      f"(aar_run_lattice)", "nmesh": N, "n_modes": M,
                          "l2": "working set >> L2 (no flush)",
                          "parallelism": "replicas" if world > 1 else "single GPU"},
               "roofline": roofline, "path_roofline": path_roof, "cpu_baseline": cpu, "e2e": e2e,
               "plain_fp64": plain.get("plain_fp64"), "plain_fp64_regrouped": plain.get("plain_fp64_regrouped"),
               "gpu_launches": launches, "clocks": clocks, "precision_vs_fp64_oracle": precision, "kernels": kernels,
               "schedule": tuned}
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


def slab_alg_bytes(name: str, N: int, S: int, M: int, R: int, npart: int) -> float:
    """Algorithmic HBM bytes of one launch of each slab-form kernel (F = one
    half-spectrum field, F_s = F / S one slab field; the accumulations
    read-modify-write the two compensated accumulator fields)."""
    F = 8.0 * N * N * (N // 2 + 1)
    Fs = F / S
    table = {
        "seedtable": 4.0 * N * N, "noise": F + 4.0 * N * N,
        "slab_fold": F + M * Fs, "slab_c2r": 2 * Fs, "slab_r2c": 2 * Fs, "slab_products": (M + R) * Fs,
        "slab_acc": R * Fs + 4 * F, "slab_combine": 4 * F,
        "slab_lpt_fold_hess": F + 6 * Fs, "slab_lpt_source": 7 * Fs, "slab_lpt_acc": Fs + 2 * F,
        "slab_lpt_fold_disp": 2 * F + 6 * Fs, "slab_scatter": 12 * Fs,
        # glass read-out: the six displacement fields once, Pos / Vel out
        "readout_glass": 6 * 4.0 * N ** 3 + 24.0 * npart,
    }
    return table.get(name, float("nan"))


def slab_arm(args):
    """The slab form (AAR_SLAB_FP32) on one GPU: the 1536^3 large single run
    (or any workload with --slab S).  Particles: the 64^3 lattice glass tiled
    N/64 times (aar_run_lattice); by default written straight into pinned host
    memory by the read-out (page-locked host buffers are device-addressable),
    so the device holds only the plan (potential, arena, FFT work area)."""
    import ctypes
    import torch
    from aarambam_gb300 import _lib
    from aarambam_gb300.ic import ICGenerator
    _lib.load(build_if_missing=True)
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    cfg = make_cfg(args.workload, 1234)
    N, M = cfg["Nmesh"], cfg["N_modes"]
    S = args.slab or SLAB_DEFAULT.get(args.workload, 8)
    alpha, x0, k, t = load_tables(cfg["table"], M)
    R = active_r(alpha)
    free0, total = torch.cuda.mem_get_info()
    gen = ICGenerator(cfg, alpha, x0, k, t, precision="slab_fp32", nslab=S)
    gen.prepare()
    gn = min(N, 64)
    tile = N // gn
    npart = N ** 3
    host = not args.slab_device_out
    t_alloc = time.perf_counter()

    def pinned(shape):
        # page-locked in place (cudaHostRegister): the caching host
        # allocator behind pin_memory rounds sizes up to powers of two
        a = torch.from_numpy(np.empty(shape, np.float32))
        rc = torch.cuda.cudart().cudaHostRegister(a.data_ptr(), a.numel() * a.element_size(), 0)
        if int(rc) != 0:
            raise RuntimeError(f"cudaHostRegister failed ({rc})")
        return a
    mk = pinned if host else (lambda shape: torch.empty(shape, dtype=torch.float32, device=dev))
    pos, vel = mk((npart, 3)), mk((npart, 3))
    t_alloc = time.perf_counter() - t_alloc

    # positions and velocities (IDs are 1-based int32 in the reference's
    # 32-bit-ID build and would pass 2^31 at 1536^3)
    def step():
        gen.run_lattice(gn, 100.0, tile, pos, vel, None)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    free_min = torch.cuda.mem_get_info()[0]
    clk = Clocks(0)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        step()
        launches += gen.launches
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    elapsed = e0.elapsed_time(e1) / 1e3
    free_min = min(free_min, torch.cuda.mem_get_info()[0])
    value = args.steps * npart / elapsed
    # per-kernel times of one profiled step
    buf = ctypes.create_string_buffer(1 << 16)
    gen.L.aar_profile_enable(gen.h, 1)
    step()
    gen.L.aar_profile_report(gen.h, buf, len(buf))
    gen.L.aar_profile_enable(gen.h, 0)
    kernels = {}
    for line in buf.value.decode().strip().splitlines():
        nm, cnt, ms = line.split(",")
        kernels[nm] = {"launches": int(cnt), "ms": float(ms)}
    tot = sum(v["ms"] for v in kernels.values())
    pk = peaks()
    for nm, v in kernels.items():
        per = v["ms"] / v["launches"] / 1e3
        v["share"] = round(v["ms"] / tot, 4)
        v["gbs"] = round(slab_alg_bytes(nm, N, S, M, R, npart) / per / 1e9, 1)
    own = [n for n in kernels if n not in ("slab_c2r", "slab_r2c")]  # cuFFT: library kernels
    dom = max(own, key=lambda n: kernels[n]["ms"])
    d_per = kernels[dom]["ms"] / kernels[dom]["launches"] / 1e3
    achieved = slab_alg_bytes(dom, N, S, M, R, npart) / d_per / 1e9
    fft_ms = sum(kernels[n]["ms"] for n in ("slab_c2r", "slab_r2c") if n in kernels)
    out_bytes = 24 * npart
    print(json.dumps({
        "metric": f"IC particles/s at {N}^3 (slab FP32 form)", "value": value, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{args.workload}: Nmesh={N}^3 particles, Box={cfg['Box']} Mpc/h, {cfg['table']} "
                               f"({M} modes, {R} active r), Fnl={cfg['Fnl']}, BBKS T(k), z=49, {gn}^3 lattice "
                               f"glass tiled {tile}^3 times (aar_run_lattice)",
                   "nmesh": N, "n_modes": M, "nslab": S, "l2": "working set >> L2 (no flush)",
                   "parallelism": "single GPU",
                   "particles": "pinned host memory, written by the read-out kernel" if host else "device buffers",
                   "plan_device_bytes": gen.device_bytes,
                   "peak_device_gb": round((total - free_min) / 1e9, 2),
                   "device_gb_before": round((total - free0) / 1e9, 2),
                   "host_alloc_s": round(t_alloc, 1)},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": None,
                     "peak_source": pk["source"]},
        "cufft_share": round(fft_ms / tot, 4),
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": out_bytes if host else 0,
                "api": "aar_run_lattice with page-locked host Pos/Vel buffers" if host else None},
        "gpu_launches": launches, "clocks": clocks, "kernels": kernels}))


def split_arm(args):
    """One realisation per step made by all ranks together: each rank
    regenerates the Gaussian potential, sums its share of the radial modes
    (balanced by product terms) and one reduce gives rank 0 the potential,
    which then runs 2LPT and the read-out (strong scaling: the work per step
    is fixed).  Time = max over ranks, CUDA events, barrier on both sides."""
    import torch
    import torch.distributed as dist
    from aarambam_gb300 import _lib, modal_split
    from aarambam_gb300.ic import ICGenerator
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 or "MASTER_ADDR" in os.environ:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load(build_if_missing=True)
    cfg = make_cfg(args.workload, 1234)
    N, M = cfg["Nmesh"], cfg["N_modes"]
    alpha, x0, k, t = load_tables(cfg["table"], M)
    gen = ICGenerator(cfg, alpha, x0, k, t)
    lagr = lattice_positions(N, cfg["Box"], dev) if rank == 0 else None
    pos = torch.empty_like(lagr) if rank == 0 else None
    vel = torch.empty_like(lagr) if rank == 0 else None
    distributed = dist.is_available() and dist.is_initialized()

    def step():
        if distributed:
            modal_split.split_run(gen, lagr, rank, world, pos=pos, vel=vel)
        else:
            gen.run(lagr, pos, vel)

    def barrier():
        torch.cuda.synchronize()
        if distributed:
            dist.barrier()
    for _ in range(args.warmup):
        step()
    barrier()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    barrier()
    el = max_over_ranks(e0.elapsed_time(e1) / 1e3, dev)
    part = modal_split.partition(alpha, world)
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": args.steps * N ** 3 / el, "unit": UNIT, "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
                          "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
                          "data": "synthetic",
                          "config": {"workload": f"{args.workload}: one realisation per step, modal sum split over "
                                                 f"{world} ranks by radial mode", "nmesh": N, "n_modes": M,
                                     "parallelism": f"modal split x{world}",
                                     "part_of_r": part.tolist()}}))
    if distributed:
        dist.destroy_process_group()


def stage_arm(args):
    """Profiling case: the plan's field stages only (no particle arrays, so
    the device holds just the plan's fields: ~7 GB at 512^3 with 12 modes)."""
    import torch
    from aarambam_gb300 import _lib
    from aarambam_gb300.ic import ICGenerator
    _lib.load(build_if_missing=True)
    torch.cuda.set_device(0)
    cfg = make_cfg(args.workload, 1234)
    alpha, x0, k, t = load_tables(cfg["table"], cfg["N_modes"])
    gen = ICGenerator(cfg, alpha, x0, k, t)
    if not args.no_autotune:
        gen.autotune()
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        for st in ("noise", "modal", "lpt"):
            gen.stage(st)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        for st in ("noise", "modal", "lpt"):
            gen.stage(st)
    e1.record(stream)
    torch.cuda.synchronize()
    print(json.dumps({"case": f"{args.workload} field stages", "ms_per_step": e0.elapsed_time(e1) / args.steps,
                      "steps": args.steps, "device_bytes": gen.device_bytes}))


def rows_arm(args):
    """Profiling case: the modal row kernel of the workload's plan (NVRTC
    kernel, 20 modes at 1024^3) on args.rows_harness rows of random fields
    with a compact field stride (aar_profile_modal_rows)."""
    import ctypes
    import torch
    from aarambam_gb300 import _lib
    from aarambam_gb300.ic import ICGenerator
    _lib.load(build_if_missing=True)
    torch.cuda.set_device(0)
    cfg = make_cfg(args.workload, 1234)
    N, M = cfg["Nmesh"], cfg["N_modes"]
    alpha, x0, k, t = load_tables(cfg["table"], M)
    R = active_r(alpha)
    gen = ICGenerator(cfg, alpha, x0, k, t)
    HP = (N // 2 + 1 + 7) // 8 * 8
    nrows = args.rows_harness
    g = torch.Generator(device="cuda").manual_seed(3)
    work = torch.randn((M + 1) * nrows * HP * 2, device="cuda", generator=g)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def once():
        _lib.check(gen.L, gen.h, gen.L.aar_profile_modal_rows(gen.h, work.data_ptr(), nrows, st))
    for _ in range(args.warmup):
        once()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        once()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    byts = (M + R) * 8.0 * nrows * HP
    print(json.dumps({"case": f"modal rows of {args.workload}, {nrows} rows", "jit": gen.jit_status,
                      "ms_per_launch": ms, "alg_bytes": byts, "gbs": byts / ms / 1e6,
                      "device_bytes": int(work.numel() * 4 + gen.device_bytes)}))


def batch_arm(args):
    """Batching workload: all realisations of the batch per step, one graph
    launch (value = particles of all realisations / step time)."""
    import torch
    from aarambam_gb300 import _lib
    from aarambam_gb300.ic import ICBatch, ICGenerator
    _lib.load(build_if_missing=True)
    nreal, N, box = BATCH_WORKLOADS[args.workload]
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    base = make_cfg("scalarI_m12_n256", 0)
    gens, bytes_step = [], 0.0
    for i in range(nreal):
        tab, M, fnl = BATCH_TEMPLATES[i % len(BATCH_TEMPLATES)]
        cfg = dict(base, Nmesh=N, Nsample=N, Nmax=256, Box=box, Seed=1234 + i, Fnl=fnl, N_modes=M, table=tab)
        alpha, x0, k, t = load_tables(tab, M)
        gens.append(ICGenerator(cfg, alpha, x0, k, t))
        bytes_step += 4.0 * N ** 3 * (46 + 9 * M)
    lagr = lattice_positions(N, box, dev)
    npart = lagr.shape[0]
    lagrs = [lagr] * nreal
    poss = [torch.empty_like(lagr) for _ in range(nreal)]
    vels = [torch.empty_like(lagr) for _ in range(nreal)]
    b = ICBatch(gens)
    for _ in range(args.warmup):
        b.run(lagrs, poss, vels)
    torch.cuda.synchronize()
    clk = Clocks(0)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        b.run(lagrs, poss, vels)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    el = e0.elapsed_time(e1) / 1e3
    # the same realisations one after another without the graph, for comparison
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for g, p, v in zip(gens, poss, vels):
        g.run(lagr, p, v)
    s1.record(stream)
    torch.cuda.synchronize()
    serial = s0.elapsed_time(s1) / 1e3
    pk = peaks()
    per = el / args.steps
    value = nreal * npart * args.steps / el
    print(json.dumps({
        "metric": f"IC particles/s, batch of {nreal} realisations at {N}^3 (fused FP32 form, one CUDA graph)",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * per, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"{args.workload}: {nreal} realisations, {N}^3, Box {box}, templates "
                               + ", ".join(f"{tb} ({m} modes)" for tb, m, _ in BATCH_TEMPLATES) + " cycled, own seeds",
                   "nmesh": N, "realisations": nreal, "l2": "working set >> L2 (no flush)"},
        "roofline": {"kernel": "whole batch graph", "bound": "hbm", "achieved": round(bytes_step / per / 1e9, 1),
                     "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": round(bytes_step / per / 1e9 / pk["hbm_gbs"], 4),
                     "traffic": None, "peak_source": pk["source"]},
        "serial_ms": 1e3 * serial, "graph_speedup_vs_serial": round(serial / per, 3),
        "gpu_launches": b.launches * args.steps, "clocks": clocks, "cpu_baseline": None, "e2e": None}))


def decomp_arm(args):
    """Modal decomposition: seconds per Decomposer.go (covariance build and
    matching pursuit on the GPU, FP64), next to the reference Decomposer's
    own time for the same table where it was made (its meta.json, measured on
    an 8-core x86 host)."""
    import torch
    from aarambam_gb300 import _lib, models, utils
    from aarambam_gb300.basis import BasicBasisDecompose
    _lib.load(build_if_missing=True)
    model, M, lbox, nmax, kw, table = DECOMP_WORKLOADS[args.workload]
    torch.cuda.set_device(0)
    dec = utils.Decomposer(M, 0.965, lbox, nmax, 1e-4, 150)
    times, out, inst = [], None, None
    for i in range(max(1, args.warmup) + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        inst = type("C", (getattr(models, model), BasicBasisDecompose), {})(**dec.args, verbose=False, **kw)
        out = inst.go()
        torch.cuda.synchronize()
        if i >= max(1, args.warmup):
            times.append(time.perf_counter() - t0)
    ref = None
    if table:
        mpath = os.path.join(TABLES, table, "meta.json")
        if os.path.exists(mpath):
            with open(mpath) as f:
                ref = json.load(f).get("seconds")
    per = sum(times) / len(times)
    print(json.dumps({
        "metric": "seconds per modal decomposition (Decomposer.go)", "value": per, "unit": "s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * per,
        "higher_is_better": False, "scaling": None, "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {model} {kw}, N_modes {M}, Lbox {lbox}, Nmax {nmax}, "
                               "k_grid_size 150, ModeTol 1e-4, MaxModeCount 150",
                   "modes": int(inst.basis.mode_indices.shape[1]), "tetrapyd_points": int(inst.basis.tetrapyd_grid_size),
                   "pursuit_steps": len(inst.basis.omp_log), "nonzero_alpha": int(np.count_nonzero(out["AlphaTable"][:, 3]))},
        "covariance_s": inst.basis.timings["covariance_s"],
        "pursuit_s": {(k[8:-2] or "total"): round(v, 4) for k, v in inst.basis.timings.items() if k.startswith("pursuit_")},
        "reference_decomposer_s": ref,
        "reference_decomposer_host": "8-core x86 (the table's meta.json)" if ref else None}))


def cov_arm(args):
    """The mode-bispectrum covariance alone (aar_tetra_covariance: FP64 mode
    values, bf16 digit tiles, the tcgen05 split-digit GEMM, the int64
    reduce), seconds per build with CUDA events on the launching stream;
    roofline against the measured bf16 tensor peak with the MMA flops the
    GEMM issues (36 digit-pair products of 128 x 64 x 16 per 16 points and
    tile pair)."""
    import ctypes as C
    import torch
    from aarambam_gb300 import _lib
    from aarambam_gb300.basis import Basis
    L = _lib.load(build_if_missing=True)
    M, lbox, nmax, kgrid = COV_WORKLOADS[args.workload]
    torch.cuda.set_device(0)
    kF = 2 * np.pi / lbox
    b = Basis(k_min=kF, k_max=kF * nmax, parameter_n_scalar=0.965, mode_p_max=M, k_grid_size=kgrid, verbose=False)
    nm, npts = b.mode_indices.shape[1], b.tetrapyd_grid_size
    nbytes = L.aar_tetra_covariance_scratch_bytes(npts, nm)
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    qq = torch.empty((nm, nm), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()

    def one():
        b._call("aar_tetra_covariance", C.c_void_p(qq.data_ptr()), *b._tetra_args(), C.c_void_p(scratch.data_ptr()),
                C.c_size_t(nbytes), C.c_void_p(st.cuda_stream))
    for _ in range(max(3, args.warmup)):
        one()
    clocks = Clocks(0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        one()
    e1.record(st)
    torch.cuda.synchronize()
    ck = clocks.stop()
    per = e0.elapsed_time(e1) / 1e3 / args.steps
    ta, tb = -(-nm // 128), -(-nm // 64)
    pairs = sum(tb - 2 * i for i in range(ta))
    nch = -(-npts // 128) * 8
    mma_flops = pairs * nch * 36 * 2.0 * 128 * 64 * 16
    pk = peaks()
    diff = np.abs(qq.cpu().numpy() - b.mode_bispectra_covariance).max()
    print(json.dumps({
        "metric": "seconds per mode-bispectrum covariance (aar_tetra_covariance)", "value": per, "unit": "s",
        "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": 1e3 * per,
        "higher_is_better": False, "scaling": None, "vs_baseline": None, "dtype": "bf16 digits, FP32 level sums, "
        "int64 fixed point (FP64-accurate)", "data": "synthetic",
        "config": {"workload": f"{args.workload}: N_modes {M} ({nm} 3D modes), Lbox {lbox}, Nmax {nmax}, "
                               f"k_grid_size {kgrid} ({npts} tetrapyd points)", "tile_pairs": pairs,
                   "l2": "operand digits far larger than L2 (no flush)"},
        "roofline": {"kernel": "whole covariance call (k_tetra_modes, k_modes_rowmax, k_tetra_digits, k_gram_tc, "
                               "k_gram_tc_reduce)",
                     "bound": "tensor", "achieved": round(mma_flops / per / 1e12, 1), "peak": pk["bf16_tflops"],
                     "unit": "TFLOP/s", "frac": round(mma_flops / per / 1e12 / pk["bf16_tflops"], 4),
                     "traffic": None, "peak_source": pk["source"]},
        "mma_flops_per_build": mma_flops, "fp64_equivalent_flops": float(nm) * (nm + 1) * npts,
        "repeat_max_abs_diff": float(diff), "clocks": ck, "gpu_launches": 5 * args.steps,
        "cpu_baseline": None, "e2e": None}))


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload not in WORKLOADS:  # batches / decompositions / covariance: the IC path's reference arm
        args.workload = "scalarI_m12_n256"
    cfg = make_cfg(args.workload, 1234)
    n = args.cpu_sample_n
    # size the sample so the whole run stays within a few minutes
    first = cpu_baseline(args.workload, n, 1)[0]
    per = n ** 3 / first["value"]
    while n > 32 and per * (args.steps + args.warmup) > 240:
        n //= 2
        first = cpu_baseline(args.workload, n, 1)[0]
        per = n ** 3 / first["value"]
    for _ in range(max(0, args.warmup - 1)):
        cpu_baseline(args.workload, n, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_baseline(args.workload, n, 1)
    el = time.perf_counter() - t0
    value = args.steps * n ** 3 / el
    base = dict(first, value=value)
    print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": 0,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                      "data": "synthetic", "config": {"workload": f"{args.workload} sampled at {n}^3",
                                                      "nmesh": cfg["Nmesh"]},
                      "cpu_baseline": base,
                      "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        reference_arm(a)
    elif a.split_modal:
        split_arm(a)
    elif a.stages_only:
        stage_arm(a)
    elif a.rows_harness:
        rows_arm(a)
    elif a.workload in BATCH_WORKLOADS:
        batch_arm(a)
    elif a.workload in DECOMP_WORKLOADS:
        decomp_arm(a)
    elif a.workload in COV_WORKLOADS:
        cov_arm(a)
    elif a.slab or a.workload in SLAB_DEFAULT:
        slab_arm(a)
    else:
        gpu_arm(a)

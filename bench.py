#!/usr/bin/env python3
"""H|psi> band-applications per second on GB300.

Workload (one "step"): H|psi> = (T + V_loc + V_NL)|psi> on a block of 128
bands of the 64-atom simple-cubic diamond supercell (a = 20.52 bohr,
Ecut 20 Ha -> 37,073 plane waves at Gamma, FFT grid 72^3, s/p/d x 2
Kleinman-Bylander projectors per atom -> 1,152 projectors), synthetic
seeded data of those shapes.  One band-application = H applied to one band.

  value  — device-resident inputs (psi, hpsi in HBM), CUDA-event timed.
  e2e    — the same call through the public API with pinned host buffers:
           H2D of psi and hpsi, compute, D2H of hpsi inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--prec fp32|fp64|tc] [--impl gb300|reference]

With --gpus N > 1 (launched under torchrun) every rank runs an independent
replica of the workload (no collective on the data path); value is the sum.
"""
import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--prec", default="tc", choices=["fp32", "fp64", "tc", "tc_bf16"])
    ap.add_argument("--system", default="sc64")
    ap.add_argument("--nb", type=int, default=128)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--serving-requests", type=int, default=10000,
                    help="requests of the served Poisson stream (0 skips serving)")
    ap.add_argument("--serving-rate", type=float, default=200.0)
    ap.add_argument("--serving-lanes", type=int, default=8)
    ap.add_argument("--serving-sweep", type=float, nargs="*", default=[250.0, 300.0, 350.0, 400.0, 500.0],
                    help="rates (req/s) of the capacity sweep after the main stream")
    ap.add_argument("--no-sternheimer", action="store_true",
                    help="skip the Sternheimer dpsi/dk solve (2-atom fcc cell, 4 occupied bands, x/y/z)")
    ap.add_argument("--no-kp", action="store_true",
                    help="skip the k.p workload (64-atom cell, 256 bands, 7 k-points, velocity + FP64 sums)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched k-point workload (fcc2 MP 6^3 x 32 + sc8 MP 4^3 x 48 bands)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, world: int) -> float:
    """The largest x over the replicas (all-reduce MAX in the process group's
    backend: a CUDA tensor for NCCL, a host tensor otherwise).  With one
    process, x itself."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_rate(units_per_rank: int, ms_per_rank: float, world: int) -> float:
    """Whole-job units/s of `world` replicas: all units over the slowest rank's time."""
    return world * units_per_rank / (max_over_ranks(ms_per_rank, world) * 1e-3)


def workload(name, nb):
    from effmass_gb300 import system as S
    sysm = S.make_system(name)
    kp = S.g_sphere(sysm.lattice, S.default_kpoint(name), sysm.ecut)
    psi = S.make_bands(kp, nb, seed=11)
    return sysm, kp, psi


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    INTERVAL_MS = 50

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def _rows(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        return rows

    def start(self):
        """Start sampling and wait (at most 5 s) for the first sample, so that the
        sampler is running when the timed region begins."""
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        t_end = time.time() + 5.0
        while time.time() < t_end and not self._rows():
            time.sleep(0.02)

    def mark(self, begin: bool):
        if begin:
            self.t0 = datetime.datetime.now()
        else:
            self.t1 = datetime.datetime.now()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        # one more interval, so that a sample follows the end of the region
        time.sleep(2 * self.INTERVAL_MS / 1000)
        self.proc.terminate()
        self.proc.wait()
        all_rows = self._rows()
        os.unlink(self.path)
        # samples inside the timed region, widened by one interval on each side
        # (a region of a few ms falls between two samples)
        rows = []
        parsed = 0
        pad = datetime.timedelta(milliseconds=self.INTERVAL_MS)
        for r in all_rows:
            try:
                t = datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f")
            except ValueError:
                continue
            parsed += 1
            if self.t0 is None or self.t1 is None or self.t0 - pad <= t <= self.t1 + pad:
                rows.append(r)
        window = "timed region +- %d ms" % self.INTERVAL_MS
        if not parsed:  # unreadable timestamps: every sample taken while sampling ran
            rows, window = all_rows, "whole sampling run"
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows), "window": window}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    return 6800.0, 1900.0, "fallback"


def nxs_of(sysm, kp):
    import numpy as np
    return int(len(np.unique(np.mod(kp.g_idx[:, 0], sysm.n1))))


def run_gb300(args, rank, world, local):
    import numpy as np
    import torch
    from effmass_gb300.hamiltonian import Hamiltonian

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    sysm, kp, psi = workload(args.system, args.nb)
    nb, npw, P = args.nb, kp.npw, sysm.n_proj_total
    H = Hamiltonian(sysm)
    H.set_kpoint(0, kp)
    psi_d = torch.from_numpy(psi).cuda()
    hpsi_d = torch.zeros_like(psi_d)
    stream = torch.cuda.current_stream()

    def step(prec):
        H.apply(0, nb, psi_d, hpsi_d, prec)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # set-up call (builds the projector matrices of this precision once)
    step(args.prec)
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        step(args.prec)
    barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.mark(True)
    e0.record(stream)
    for _ in range(args.steps):
        step(args.prec)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.mark(False)
    clk = clocks.stop()
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world)
    value = replicas_rate(nb, ms, world)

    # per-phase CUDA-event profile over the same number of steps, with the
    # tensor-core projection chain on the launching stream (HPSI_ONE_STREAM):
    # on its side stream its events would also count the time it waits for
    # SMs behind the FFT passes
    H.profile(True)
    for _ in range(args.steps):
        H.apply(0, nb, psi_d, hpsi_d, args.prec, one_stream=True)
    prof = H.profile_read()
    H.profile(False)
    launches = sum(n for _, n in prof.values())
    gpu_launches = launches  # our kernels in `steps` profiled steps == the timed region's count

    # accuracy of this path against the FP64 GPU path on the same bands
    nchk = min(nb, 16)
    h64 = torch.zeros((nchk, npw), dtype=torch.complex128, device="cuda")
    hmx = torch.zeros_like(h64)
    H.apply(0, nchk, psi_d[:nchk].contiguous(), h64, "fp64")
    H.apply(0, nchk, psi_d[:nchk].contiguous(), hmx, args.prec)
    err = float(torch.linalg.norm(hmx - h64) / torch.linalg.norm(h64))
    # band energies <psi|H|psi> (FP64 sums) of the mixed path vs FP64
    e_mx = torch.einsum("bg,bg->b", psi_d[:nchk].conj(), hmx).real
    e_64 = torch.einsum("bg,bg->b", psi_d[:nchk].conj(), h64).real
    de = float((e_mx - e_64).abs().max())
    # band energies through hpsi_apply_energies (FP64 reductions on the device,
    # Parseval-normalised local energy), all nb bands, against its FP64 path
    e_all = torch.zeros(nb, dtype=torch.float64, device="cuda")
    h_e = torch.zeros_like(psi_d)
    H.apply_energies(0, nb, psi_d, h_e, args.prec, e=e_all)
    e_all64 = H.apply_energies(0, nb, psi_d, torch.zeros_like(psi_d), "fp64")
    de_api = float((e_all - e_all64).abs().max())
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(args.steps):
        H.apply_energies(0, nb, psi_d, h_e, args.prec, e=e_all)
    g1.record(stream)
    torch.cuda.synchronize()
    ms_e = g0.elapsed_time(g1) / args.steps
    energies = {"api": "hpsi_apply_energies (H|psi> + FP64 band energies)", "bands": nb,
                "max_abs_diff_vs_fp64_Ha": de_api, "value": nb / (ms_e * 1e-3), "unit": "band-apps/s",
                "ms_per_step": ms_e}
    del h_e
    # charge density of the same bands (G->r only), complex64 transforms
    occ_d = torch.full((nb,), 2.0, dtype=torch.float64, device="cuda")
    rho_d = torch.zeros((sysm.n1, sysm.n2, sysm.n3), dtype=torch.float64, device="cuda")
    H.density(0, nb, psi_d, occ_d, rho=rho_d, precision="fp32")
    torch.cuda.synchronize()
    g0.record(stream)
    for _ in range(args.steps):
        H.density(0, nb, psi_d, occ_d, rho=rho_d, precision="fp32")
    g1.record(stream)
    torch.cuda.synchronize()
    ms_d = g0.elapsed_time(g1) / args.steps
    density = {"api": "hpsi_density (complex64 G->r, compensated FP32 sums per 8 bands, FP64 across them)", "bands": nb,
               "value": nb / (ms_d * 1e-3), "unit": "band-densities/s", "ms_per_step": ms_d}
    del rho_d

    fp64 = None
    if not args.no_fp64 and args.prec != "fp64":
        step("fp64")
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 2
        f0.record(stream)
        for _ in range(reps):
            step("fp64")
        f1.record(stream)
        torch.cuda.synchronize()
        fp64 = nb / (f0.elapsed_time(f1) / reps * 1e-3)

    # dH/dk_{x,y,z}|psi> on the same block (the 64-atom workload asks for it beside H|psi>)
    from effmass_gb300.hamiltonian import GradHPsi
    gx, gy, gz = (torch.zeros_like(psi_d) for _ in range(3))
    gout = GradHPsi(gx, gy, gz)
    H.grad_apply(0, nb, psi_d, gout, args.prec)
    torch.cuda.synchronize()
    q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    q0.record(stream)
    for _ in range(args.steps):
        H.grad_apply(0, nb, psi_d, gout, args.prec)
    q1.record(stream)
    torch.cuda.synchronize()
    grad_value = replicas_rate(nb, q0.elapsed_time(q1) / args.steps, world)
    del gx, gy, gz, gout

    # end to end through the public API with pinned host buffers
    psi_h = torch.from_numpy(psi).pin_memory()
    hpsi_h = torch.zeros_like(psi_h).pin_memory()
    psi_np, hpsi_np = psi_h.numpy(), hpsi_h.numpy()
    for _ in range(max(1, args.warmup)):
        H.apply(0, nb, psi_np, hpsi_np, args.prec)
    dstream = torch.cuda.default_stream()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    g0.record(dstream)
    for _ in range(args.steps):
        H.apply(0, nb, psi_np, hpsi_np, args.prec)
    g1.record(dstream)
    torch.cuda.synchronize()
    e2e = {"value": replicas_rate(nb, g0.elapsed_time(g1) / args.steps, world), "unit": "band-apps/s",
           "h2d_bytes_per_step": 2 * psi.nbytes, "d2h_bytes_per_step": psi.nbytes}

    # roofline of the dominant phase
    hbm, bf16, src = peaks()
    csz = 16 if args.prec == "fp64" else 8
    nxs = nxs_of(sysm, kp)
    plane = nxs * sysm.n2 * sysm.n3 * csz
    steps = args.steps
    N = sysm.n1 * sysm.n2 * sysm.n3
    alg = {
        # bytes the pass must move per step (band block): g2r reads psi (16 B per
        # G) and writes the sphere planes of T; the x pass reads and writes them
        # (+ V once); r2g reads them, psi and the kinetic energies (8 B) and, on
        # the tensor-core path, writes the complex64 local term (8 B) that the
        # expansion adds into hpsi, else reads and writes hpsi (2 x 16 B)
        "g2r_planes": ("hbm", steps * nb * (npw * 16 + plane)),
        "x_pass": ("hbm", steps * (nb * 2 * plane + N * csz // 2)),
        "r2g_planes": ("hbm", steps * nb * (plane + npw * (16 + 8 + (8 if args.prec.startswith("tc") else 32)))),
        # algorithmic flops: 8 real flops per complex multiply-add
        "proj_gemm": ("tensor", steps * 8.0 * P * npw * nb),
        "expand_gemm": ("tensor", steps * 8.0 * P * npw * nb),
    }
    dom = max((k for k in alg), key=lambda k: prof[k][0])
    bound, work = alg[dom]
    tms = prof[dom][0]
    if bound == "hbm":
        ach = work / (tms * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "peak_source": src}
    else:
        ach = work / (tms * 1e-3) / 1e12
        roof = {"bound": "tensor", "kernel": dom, "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
                "frac": ach / bf16, "peak_source": src + " dense bf16 tensor peak"}
    # DRAM bytes (read + write) of one launch of this workload (128 bands per
    # launch, 64-atom cell, split-FP16 tensor-core path) from ncu --set full
    # captures of this bench command: x pass 219.2 + 156.7 MB, G->r planes
    # 76.3 + 160.5 MB, r->G planes 294.2 + 29.1 MB, projection GEMM 98.2 +
    # 13.1 MB, expansion GEMM 138.4 + 25.7 MB (cold caches: ncu flushes them
    # between passes)
    ncu_traffic = {"x_pass": 375.91e6, "g2r_planes": 236.75e6, "r2g_planes": 323.32e6, "proj_gemm": 111.3e6,
                   "expand_gemm": 164.1e6}
    roof["traffic"] = ncu_traffic.get(dom) if (args.system == "sc64" and args.prec == "tc") else None
    if roof["traffic"] is not None and bound == "hbm":
        roof["algorithmic_bytes_per_launch"] = alg[dom][1] / prof[dom][1]
        roof["traffic_note"] = "ncu dram__bytes_read+write of one launch; below the algorithmic bytes because " \
                               "part of the launch's writes are still in the 129 MB L2 when it ends"
    elif roof["traffic"] is not None:
        roof["traffic_note"] = "ncu dram__bytes_read+write of one launch: the band operand and hpsi / the " \
                               "local term the epilogue reads and writes; the projector tiles are generated " \
                               "in shared memory and add no DRAM traffic"
    # the tensor-core projection GEMM, reported beside the dominant phase
    roof_gemm = None
    if prof["proj_gemm"][1]:
        t_g = prof["proj_gemm"][0]
        a_g = alg["proj_gemm"][1] / (t_g * 1e-3) / 1e12
        roof_gemm = {"bound": "tensor", "kernel": "proj_gemm", "achieved": a_g, "peak": bf16, "unit": "TFLOP/s",
                     "frac": a_g / bf16, "peak_source": src + " dense bf16 tensor peak",
                     "note": "algorithmic flops 8*P*npw*nb; the split operands issue 3x that on the tensor pipe"}
    # the whole local term (the three FFT passes) on its canonical bytes per
    # band, 3 N s_c + 3 npw s_c, plus V (4 or 8 B per grid point) once per band block
    roof_local = None
    loc = [k for k in ("g2r_planes", "x_pass", "r2g_planes") if prof.get(k, (0, 0))[1]]
    if len(loc) == 3:
        t_l = sum(prof[k][0] for k in loc)
        b_l = steps * (nb * (3 * N * csz + 3 * npw * csz) + N * csz // 2)
        a_l = b_l / (t_l * 1e-3) / 1e9
        roof_local = {"bound": "hbm", "kernels": loc, "achieved": a_l, "peak": hbm, "unit": "GB/s",
                      "frac": a_l / hbm, "peak_source": src, "bytes_per_band": b_l / (steps * nb),
                      "ms_per_step": t_l / steps}
    phases = {k: {"ms_per_step": v[0] / steps, "launches_per_step": v[1] / steps} for k, v in prof.items() if v[1]}

    serving = None
    if args.serving_requests > 0:
        serving = run_serving(args, H, kp)
    batched = None
    if rank == 0 and not args.no_batched:
        batched = run_batched(args)
    kp_out = None
    if rank == 0 and not args.no_kp:
        kp_out = run_kp(args)
    stern = None
    if rank == 0 and not args.no_sternheimer:
        stern = run_sternheimer(args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import cpu_baseline
        cpu = cpu_baseline.run(sysm, kp, psi[:16], bands_per_worker=2)
        cpu = {"value": cpu["value"], "unit": "band-apps/s", "cores": cpu["cores"], "kind": cpu["kind"],
               "sample": cpu["sample"], "per_core_value": cpu["per_core_value"], "cpu": cpu["cpu"]}

    out = {
        "metric": "H|psi> band-applications/s (mixed precision, rel. err <= 1e-6 vs FP64)",
        "value": value, "unit": "band-apps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "c64/f32", "fp64": "c128/f64", "tc": "c64/f32 FFT + fp16x2-split tensor (3 products, f32 acc)",
                  "tc_bf16": "c64/f32 FFT + bf16x2-split tensor (3 products, f32 acc)"}[args.prec],
        "precision_path": args.prec,
        "data": "synthetic (seeded psi, V_loc, KB projectors of the named shapes)",
        "config": {"workload": f"{args.system}: 64-atom SC diamond, 72^3 grid, Ecut 20 Ha, Gamma",
                   "npw": npw, "fft_grid": [sysm.n1, sysm.n2, sysm.n3], "bands_per_step": nb, "projectors": P,
                   "parallelism": "replicas" if world > 1 else "1 GPU",
                   "l2": "inputs larger than L2 (psi %d MB and hpsi %d MB per step, FFT planes %d MB per pass%s)"
                         % (psi.nbytes >> 20, psi.nbytes >> 20, (nb * plane) >> 20,
                            "; projector tiles generated in shared memory" if args.prec.startswith("tc")
                            else ", projector matrix %d MB" % (P * npw * csz >> 20))},
        "rel_err_vs_fp64": err, "band_energy_max_abs_diff_Ha": de_api,
        "rayleigh_quotient_of_hpsi_max_abs_diff_Ha": de, "band_energies": energies, "density": density,
        "fp64_value": fp64, "speedup_vs_fp64": (value / world / fp64) if fp64 else None,
        "grad_value": grad_value, "grad_unit": "band-apps/s of dH/dk_{x,y,z}|psi> (all three directions)",
        "e2e": e2e, "roofline": roof, "roofline_gemm": roof_gemm, "roofline_local": roof_local, "phases": phases,
        "gpu_launches": gpu_launches,
        "cpu_baseline": cpu, "clocks": clk, "serving": serving, "batched": batched, "kp": kp_out, "sternheimer": stern,
    }
    if rank == 0:
        print(json.dumps(out))
    H.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def _serving_stream(rng, n, rate, pools):
    """n seeded requests of the served mix: Poisson arrivals at `rate` req/s,
    cells 6:3:1 (2-, 8-, 64-atom), 1-16 k-points drawn from the cell's pool,
    8-128 bands."""
    import numpy as np
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
    kinds = rng.choice(3, size=n, p=[0.6, 0.3, 0.1])
    plans = []
    for i in range(n):
        si = int(kinds[i])
        nkr = int(rng.integers(1, 17))
        ks = rng.integers(0, len(pools[si][1]), size=nkr)
        nb = int(rng.integers(8, 129))
        plans.append((si, [int(k) for k in ks], nb))
    return arrivals, kinds, plans


def _serve(srv, bufs, pools, arrivals, plans):
    """Submit the stream on its arrival times from a thread, wait for every
    request; returns (per-request times, wall seconds)."""
    import threading
    from effmass_gb300.serving import Job
    n = len(plans)
    tickets = [None] * n
    t0 = time.perf_counter()

    def submitter():
        for i, (si, ks, nb) in enumerate(plans):
            delay = t0 + arrivals[i] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            ins, outs, vels = bufs[si]
            jobs = []
            for k in ks:
                npw = pools[si][1][k].npw
                jobs.append(Job(si, k, ins[: nb * npw].reshape(nb, npw), outs[: nb * npw].reshape(nb, npw),
                                vels[: 3 * nb * nb].reshape(3, nb, nb)))
            tickets[i] = srv.submit(jobs)

    th = threading.Thread(target=submitter)
    th.start()
    times = []
    for i in range(n):
        while tickets[i] is None:
            time.sleep(0.0002)
        times.append(srv.wait(tickets[i]))
    th.join()
    return times, time.perf_counter() - t0


def run_serving(args, H_sc64, kp_sc64):
    """Served stream (the C4 workload): Poisson arrivals at --serving-rate of
    --serving-requests requests mixing the 2-, 8- and 64-atom cells (6:3:1),
    each 1-16 k-points x 8-128 bands of H|psi> plus the velocity matrix, over
    the full k-point pools (the 216 k-points of the fcc cell's 6^3
    Monkhorst-Pack grid, the 64 of the 8-atom cell's 4^3 grid, 4 k-points of
    the 64-atom cell), through the library's serving loop.  Then a capacity
    sweep: the same mix at higher rates; the capacity is the highest rate whose
    completed throughput keeps up with the offered one (>= 95%) with p99 below
    250 ms.  Returns the summary dict."""
    import numpy as np
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    from effmass_gb300.serving import Job, Server, pinned_empty

    rng = np.random.default_rng(2024)
    pools = []
    made = []
    for name, grid in (("fcc2", 6), ("sc8", 4)):
        sysm = S.make_system(name)
        H = Hamiltonian(sysm)
        kps = []
        for i, k in enumerate(S.mp_grid(grid)):
            kp = S.g_sphere(sysm.lattice, k, sysm.ecut)
            H.set_kpoint(i, kp)
            kps.append(kp)
        made.append(H)
        pools.append((H, kps))
    # the 64-atom cell: Gamma (slot 0, already bound) and three more k-points
    sc64_k = [kp_sc64]
    sysm64 = S.make_system("sc64")
    for i, k in enumerate([(0.01, 0.0, 0.0), (0.0, 0.01, 0.0), (0.0, 0.0, 0.01)]):
        kp = S.g_sphere(sysm64.lattice, k, sysm64.ecut)
        H_sc64.set_kpoint(1 + i, kp)
        sc64_k.append(kp)
    pools.append((H_sc64, sc64_k))
    hams = [p[0] for p in pools]
    # pinned host buffers per cell (128 bands of its largest sphere), shared by
    # all requests of the cell: the stream measures time, not results
    bufs = []
    for H, kps in pools:
        npw_max = max(kp.npw for kp in kps)
        ins = pinned_empty((128 * npw_max,))
        ins[:] = 0.0
        ins[: 128 * kps[0].npw] = S.make_bands(kps[0], 128, seed=int(rng.integers(1 << 30))).ravel()
        bufs.append((ins, pinned_empty((128 * npw_max,)), pinned_empty((3 * 128 * 128,))))
    cfg = dict(lanes=args.serving_lanes, budget_gb=64, precision=args.prec, merge_max_bands=1024, bypass_ms=20.0)

    def summary(times, kinds, plans, wall, rate, last_arrival_s):
        tot = np.array([t["total_ms"] for t in times])
        que = np.array([t["queue_ms"] for t in times])
        band_apps = sum(len(p[1]) * p[2] for p in plans)
        by_kind = {}
        for name, kd in (("fcc2", 0), ("sc8", 1), ("sc64", 2)):
            sel = tot[kinds == kd]
            if sel.size:
                by_kind[name] = {"requests": int(sel.size), "p50_ms": float(np.percentile(sel, 50)),
                                 "p99_ms": float(np.percentile(sel, 99))}
        offered = len(plans) / last_arrival_s
        return {"requests": len(plans), "rate_req_per_s": rate, "band_apps": int(band_apps), "wall_s": wall,
                "throughput_band_apps_per_s": band_apps / wall, "throughput_req_per_s": len(plans) / wall,
                "offered_req_per_s": offered, "p50_ms": float(np.percentile(tot, 50)),
                "p99_ms": float(np.percentile(tot, 99)), "max_ms": float(tot.max()),
                "mean_queue_ms": float(que.mean()), "by_cell": by_kind}

    with Server(hams, **cfg) as srv:
        # warm-up: a few requests per system
        for si in range(3):
            ins, outs, vels = bufs[si]
            npw = pools[si][1][0].npw
            for _ in range(3):
                srv.wait(srv.submit([Job(si, 0, ins[: 8 * npw].reshape(8, npw), outs[: 8 * npw].reshape(8, npw),
                                         vels[: 3 * 64].reshape(3, 8, 8))]))
        n = args.serving_requests
        arrivals, kinds, plans = _serving_stream(rng, n, args.serving_rate, pools)
        times, wall = _serve(srv, bufs, pools, arrivals, plans)
        out = summary(times, kinds, plans, wall, args.serving_rate, float(arrivals[-1]))
        st = srv.stats()
        out.update({"lanes": args.serving_lanes, "precision": args.prec, "merge_max_bands": cfg["merge_max_bands"],
                    "bypass_ms": cfg["bypass_ms"], "units": st["units"], "merged_units": st["merged_units"],
                    "merged_jobs": st["merged_jobs"], "peak_device_bytes": st["peak_bytes"],
                    "mix": "2-, 8-, 64-atom cells 6:3:1; 1-16 k-points (pools of 216/64/4) x 8-128 bands; "
                           "H|psi> + velocity matrix"})
        # capacity sweep: the same mix at higher rates, fewer requests each
        sweep = []
        capacity = args.serving_rate if (out["throughput_req_per_s"] >= 0.95 * out["offered_req_per_s"]
                                         and out["p99_ms"] < 250.0) else None
        for rate in args.serving_sweep:
            if rate <= args.serving_rate:
                continue
            m = max(200, min(n, int(rate * 8)))
            a2, k2, p2 = _serving_stream(rng, m, rate, pools)
            t2, w2 = _serve(srv, bufs, pools, a2, p2)
            s2 = summary(t2, k2, p2, w2, rate, float(a2[-1]))
            keeps_up = s2["throughput_req_per_s"] >= 0.95 * s2["offered_req_per_s"] and s2["p99_ms"] < 250.0
            sweep.append({k: s2[k] for k in ("rate_req_per_s", "requests", "throughput_req_per_s",
                                             "throughput_band_apps_per_s", "p50_ms", "p99_ms")} |
                         {"keeps_up": keeps_up})
            if keeps_up:
                capacity = rate
            else:
                break
        out["capacity_sweep"] = sweep
        out["capacity_req_per_s"] = capacity
        out["capacity_rule"] = "highest swept rate with completed >= 95% of offered req/s and p99 < 250 ms"
    for H in made:
        H.close()
    return out


def batched_cells():
    """The batched k-point workload: the 2-atom fcc cell on a 6x6x6 Monkhorst-Pack
    grid with 32 bands per k-point and the 8-atom cubic cell on a 4x4x4 grid with
    48 bands; seeded orthonormal psi per k-point."""
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian
    cells = []
    for ci, (name, m, nb) in enumerate((("fcc2", 6, 32), ("sc8", 4, 48))):
        sysm = S.make_system(name)
        H = Hamiltonian(sysm)
        kps = [S.g_sphere(sysm.lattice, k, sysm.ecut) for k in S.mp_grid(m)]
        psis = []
        for i, kp in enumerate(kps):
            H.set_kpoint(i, kp)
            psis.append(S.make_bands(kp, nb, seed=1000 * ci + i))
        cells.append((name, sysm, H, kps, nb, psis))
    return cells


def run_batched(args):
    """All k-points of both cells in one graph-launched plan (FP32, tensor-core
    and FP64), against a per-k-point loop of hpsi_apply on the same device data."""
    import numpy as np
    import torch
    from effmass_gb300.batch import Batch
    from effmass_gb300.serving import pinned_empty
    cells = batched_cells()
    items = [(H, i, nb) for (_, _, H, kps, nb, _) in cells for i in range(len(kps))]
    psis = [p for c in cells for p in c[5]]
    band_apps = sum(nb for _, _, nb in items)
    steps, warm = max(args.steps, 5), max(args.warmup, 3)
    stream = torch.cuda.current_stream()

    def ev_time(fn, n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    res, outs, infos = {}, {}, {}
    for prec in ("fp32", "tc", "fp64"):
        t0 = time.perf_counter()
        plan = Batch(items, precision=prec)
        create_s = time.perf_counter() - t0
        psi_h = pinned_empty((plan.n_complex,))
        plan.pack(psis, psi_h)
        hpsi_h = pinned_empty((plan.n_complex,))
        hpsi_h[:] = 0
        plan.apply(psi_h, hpsi_h)  # leaves psi resident in the plan's buffers
        outs[prec] = np.array(hpsi_h)
        ms = ev_time(lambda: plan.run(stream), steps)
        # end to end: pinned host psi/hpsi copied in and hpsi copied out every step
        for _ in range(warm):
            plan.apply(psi_h, hpsi_h)
        t0 = time.perf_counter()
        for _ in range(steps):
            plan.apply(psi_h, hpsi_h)
        e2e_ms = (time.perf_counter() - t0) * 1e3 / steps
        infos[prec] = plan.info()
        res[prec] = {"ms_per_run": ms, "value": band_apps / (ms * 1e-3), "e2e_value": band_apps / (e2e_ms * 1e-3),
                     "create_s": create_s, "n_complex": plan.n_complex}
        if prec == "fp32":
            eager = Batch(items, precision=prec, graph=False)  # tiles come from the tuning cache
            eager.apply(psi_h, hpsi_h)
            res[prec]["eager_ms_per_run"] = ev_time(lambda: eager.run(stream), steps)
            eager.close()
            # per-k-point calls of the unbatched API on device buffers
            tp = [torch.from_numpy(p).cuda() for p in psis]
            th = [torch.zeros_like(t) for t in tp]

            def per_k():
                for (H, kid, nb), a, b in zip(items, tp, th):
                    H.apply(kid, nb, a, b, "fp32")
            res[prec]["per_k_ms_per_run"] = ev_time(per_k, 2)
            del tp, th
        plan.close()
    a64 = outs["fp64"]

    def accuracy(a):
        """relative 2-norm error against the FP64 plan and the largest band-energy
        difference <psi_n|H|psi_n> (FP64 sums on the host)"""
        de, off = 0.0, 0
        for p in psis:
            n = p.size
            e = np.einsum("bg,bg->b", p.conj(), a[off:off + n].reshape(p.shape)).real
            e64 = np.einsum("bg,bg->b", p.conj(), a64[off:off + n].reshape(p.shape)).real
            de = max(de, float(np.abs(e - e64).max()))
            off += n
        return float(np.linalg.norm(a - a64) / np.linalg.norm(a64)), de
    err, de = accuracy(outs["fp32"])
    err_tc, de_tc = accuracy(outs["tc"])
    # local-term roofline per cell from the tuner's event timing of the three FFT launches:
    # algorithmic bytes per band 3*N*8 + 3*npw*8 (complex64 grid passes, psi read, hpsi read+write)
    hbm, _, src = peaks()
    roof = []
    for (name, sysm, H, kps, nb, _), cinfo in zip(cells, infos["fp32"]["cells"]):
        N = sysm.n1 * sysm.n2 * sysm.n3
        byts = sum(nb * (3 * N * 8 + 3 * kp.npw * 8) for kp in kps)
        ach = byts / (cinfo["timed"]["local_ms"] * 1e-3) / 1e9
        roof.append({"cell": name, "local_ms": cinfo["timed"]["local_ms"], "achieved_GBps": ach, "peak": hbm,
                     "frac": ach / hbm, "peak_source": src})
    for c in cells:
        c[2].close()
    r32 = res["fp32"]
    return {
        "workload": "fcc2 (2-atom fcc, 24^3, Ecut 15 Ha) on MP 6x6x6 = 216 k x 32 bands + sc8 (8-atom SC, 36^3, "
                    "Ecut 17.5 Ha) on MP 4x4x4 = 64 k x 48 bands",
        "band_apps_per_run": band_apps, "kpoints": len(items),
        "npw_range": {c[0]: [min(k.npw for k in c[3]), max(k.npw for k in c[3])] for c in cells},
        "value": r32["value"], "unit": "band-apps/s", "ms_per_run": r32["ms_per_run"],
        "e2e_value": r32["e2e_value"], "fp64_value": res["fp64"]["value"],
        "speedup_vs_fp64": r32["value"] / res["fp64"]["value"],
        "tc": {"value": res["tc"]["value"], "ms_per_run": res["tc"]["ms_per_run"], "e2e_value": res["tc"]["e2e_value"],
               "rel_err_vs_fp64": err_tc, "band_energy_max_abs_diff_Ha": de_tc,
               "nonlocal_ms_proj_exp": {"%dx%dx%d" % tuple(c["grid"]): [c["timed"]["proj_ms"], c["timed"]["exp_ms"]]
                                        for c in infos["tc"]["cells"]},
               "note": "nonlocal term as ragged tcgen05 GEMMs (split FP16, generated projector tiles)"},
        "eager_ms_per_run": r32["eager_ms_per_run"], "per_k_api_ms_per_run": r32["per_k_ms_per_run"],
        "rel_err_fp32_vs_fp64": err, "band_energy_max_abs_diff_Ha": de,
        "plan_create_s": {k: v["create_s"] for k, v in res.items()},
        "gpu_launches_per_run": 6 * len(cells), "tuned": infos["fp32"], "local_roofline": roof,
        "timing": "CUDA events over %d graph launches on resident buffers (psi %d MB > L2)" % (
            steps, r32["n_complex"] * 16 >> 20),
    }


def run_kp(args):
    """k.p effective-mass matrix elements: the 64-atom cell with 256 bands at 7
    k-points (Gamma and Gamma +- delta along x, y, z, delta = 0.01 * 2 pi / a),
    seeded orthonormal psi and band energies sorted uniform in [-0.5, 0.8] Ha;
    <psi_m|dH/dk_a|psi_n> for all band pairs on the tensor cores and the FP64
    sums over energy denominators for the lowest 8 bands."""
    import numpy as np
    import torch
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import Hamiltonian, kp_sums
    nb, n_low = 256, 8
    sysm = S.make_system("sc64")
    d = 0.01  # fractional: the reciprocal vectors of the cubic cell are 2 pi / a
    kpts = [(0.0, 0.0, 0.0)] + [tuple(sg * d if i == ax else 0.0 for i in range(3)) for ax in range(3)
                                for sg in (1, -1)]
    H = Hamiltonian(sysm)
    psis = []
    for i, k in enumerate(kpts):
        kp = S.g_sphere(sysm.lattice, k, sysm.ecut)
        H.set_kpoint(i, kp)
        psis.append(torch.from_numpy(S.make_bands(kp, nb, seed=700 + i)).cuda())
    E = torch.from_numpy(np.sort(np.random.default_rng(77).uniform(-0.5, 0.8, nb))).cuda()
    stream = torch.cuda.current_stream()
    M = [torch.zeros((3, nb, nb), dtype=torch.complex128, device="cuda") for _ in kpts]

    def run_all(prec):
        out = []
        for i in range(len(kpts)):
            H.velocity_matrix(i, nb, psis[i], out=M[i], precision=prec)
            out.append(kp_sums(M[i], E, n_low))
        return out

    run_all("tc")  # set-up: projector and tensor-core operands of every k-point
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 2
    e0.record(stream)
    for _ in range(reps):
        sums = run_all("tc")
    e1.record(stream)
    torch.cuda.synchronize()
    ms_all = e0.elapsed_time(e1) / reps
    Mtc = [m.clone() for m in M]
    # FP64 reference of every k-point (velocity and sums)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    sums64 = run_all("fp64")
    f1.record(stream)
    torch.cuda.synchronize()
    ms64 = f0.elapsed_time(f1)
    rel = max(float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) for a, b in zip(Mtc, M))
    ds = max(float((a[0] - b[0]).abs().max() / b[0].abs().max()) for a, b in zip(sums, sums64))
    npw = [H.dim(i) for i in range(len(kpts))]
    flops = sum(3 * 8.0 * nb * nb * n for n in npw)  # psi^H (dH psi) algorithmic flops
    H.close()
    inv_mass = [(np.eye(3) + 2 * s[0][n].cpu().numpy()).diagonal().tolist() for s in sums[:1] for n in range(2)]
    return {
        "workload": "sc64 (64-atom SC diamond, 72^3, Ecut 20 Ha), 256 bands x 7 k (Gamma, Gamma +- 0.01 2pi/a x,y,z)",
        "ms_all_kpoints": ms_all, "ms_per_kpoint": ms_all / len(kpts), "fp64_ms_all_kpoints": ms64,
        "speedup_vs_fp64": ms64 / ms_all,
        "velocity_gemm_flops_per_kpoint": flops / len(kpts),
        "velocity_tflops_incl_gradient": flops / (ms_all * 1e-3) / 1e12,
        "rel_err_velocity_tc_vs_fp64": rel, "kp_sums_max_rel_diff_tc_vs_fp64": ds,
        "n_low": n_low, "example_inverse_mass_diag_gamma_bands_0_1": inv_mass,
        "note": "each k-point: dH/dk_{x,y,z}|psi> (tensor-core projector GEMMs) + psi^H G_a on the tensor cores "
                "(split FP16, FP32 accumulation, FP64 split-K sums) + FP64 k.p sums; timed with CUDA events",
    }


def run_sternheimer(args):
    """dpsi/dk of the 4 occupied bands of the 2-atom fcc cell (Ecut 15 Ha, 24^3,
    k = (0.1, 0.2, 0.3)) by the batched CG, x/y/z, in FP64 and with the
    tensor-core H, against the exact sum over states of a dense FP64
    diagonalisation (the k-point's full H matrix, npw columns)."""
    import numpy as np
    from effmass_gb300 import system as S
    from effmass_gb300.hamiltonian import GradHPsi, Hamiltonian
    nv = 4
    sysm = S.make_system("fcc2")
    kp = S.g_sphere(sysm.lattice, (0.1, 0.2, 0.3), sysm.ecut)
    npw = kp.npw
    out = {"workload": f"fcc2, k=(0.1,0.2,0.3), npw {npw}, {nv} occupied bands, directions x,y,z"}
    with Hamiltonian(sysm) as H:
        H.set_kpoint(0, kp)
        eye = np.eye(npw, dtype=np.complex128)
        hm = np.zeros_like(eye)
        H.apply(0, npw, eye, hm, "fp64")
        hm = hm.T
        E, V = np.linalg.eigh(0.5 * (hm + hm.conj().T))
        psi = np.ascontiguousarray(V[:, :nv].T)
        d = np.zeros((3, nv, npw), dtype=np.complex128)
        H.grad_apply(0, nv, psi, GradHPsi(d[0], d[1], d[2]))
        Vc = V[:, nv:]
        for prec, tol in (("fp64", 1e-10), ("tc", 1e-6)):
            errs, its, ms = [], [], []
            for a in range(3):
                coef = Vc.conj().T @ d[a].T
                x_ref = -(Vc @ (coef / (E[nv:, None] - E[None, :nv]))).T
                H.sternheimer(0, psi, E[:nv], a, tol=tol, precision=prec)  # warm
                t0 = time.perf_counter()
                x, it, _ = H.sternheimer(0, psi, E[:nv], a, tol=tol, precision=prec)
                ms.append((time.perf_counter() - t0) * 1e3)
                its.append(it)
                errs.append(float(np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)))
            out[prec] = {"tol": tol, "iterations": its, "ms_per_solve": ms, "rel_err_vs_sum_over_states": max(errs),
                         "band_apps_per_s": float(sum(its) * nv / (sum(ms) * 1e-3))}
    out["note"] = "host-timed solves (one H application of the 4 bands, projections and FP64 dots per iteration)"
    return out


def run_reference(args, rank, world, local):
    if rank != 0:
        return
    from oracle import cpu_baseline
    sysm, kp, psi = workload(args.system, 16)
    workers = os.cpu_count() or 1
    vals, secs = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        r = cpu_baseline.run(sysm, kp, psi, bands_per_worker=1, workers=workers)
        if i >= args.warmup:
            vals.append(r["value"])
            secs.append(time.perf_counter() - t0)
    v = statistics.mean(vals)
    out = {"metric": "H|psi> band-applications/s (mixed precision, rel. err <= 1e-6 vs FP64)", "impl": "reference",
           "value": v, "unit": "band-apps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * statistics.mean(secs), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "c128/f64", "data": "synthetic",
           "config": {"workload": f"{args.system}: 64-atom SC diamond, 72^3 grid, Ecut 20 Ha, Gamma", "npw": kp.npw,
                      "fft_grid": [sysm.n1, sysm.n2, sysm.n3], "projectors": sysm.n_proj_total},
           "cpu_baseline": {"value": v, "unit": "band-apps/s", "cores": workers, "kind": r["kind"],
                            "sample": r["sample"], "per_core_value": r["per_core_value"], "cpu": r["cpu"]},
           "e2e": {"value": v, "unit": "band-apps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_gb300(args, rank, world, local)


if __name__ == "__main__":
    main()

"""Timed CPU baseline of H|psi> on the host cores — TEST INFRASTRUCTURE.

Runs the reference's own H|psi> (oracle/_ref/ref_bench, built from the
reference sources at -O3) as one single-threaded process per core — the reference
is single-threaded — over independent bands of the same k-point.  If the
reference driver cannot be built on this machine, the oracle port
(oracle/hpsi_oracle.c) runs instead on the same number of threads.

Only bench.py's CPU-baseline legs use this module.
"""
from __future__ import annotations

import json
import os
import platform
import statistics
import subprocess
import tempfile
import time

from effmass_gb300 import system as S
from oracle import oracle as O


def cpu_model() -> str:
    """The host CPU's name from /proc/cpuinfo (model name, else the Arm part
    number), with the machine type."""
    name = ""
    try:
        for line in open("/proc/cpuinfo"):
            key, _, val = line.partition(":")
            key = key.strip().lower()
            if key == "model name" and val.strip():
                name = val.strip()
                break
            if key == "cpu part" and not name:
                name = "CPU part " + val.strip()
    except OSError:
        pass
    return f"{name or 'unknown'} ({platform.machine()}, {os.cpu_count()} logical CPUs)"


def run(sysm, kp, psi, bands_per_worker: int = 2, workers: int = 0):
    """Returns dict(value=band-apps/s of all workers, per_core_value=band-apps/s
    of one single-threaded worker while all run, cores, kind, sample, seconds,
    cpu)."""
    workers = workers or os.cpu_count() or 1
    nb = psi.shape[0]
    if O.build_ref():
        with tempfile.TemporaryDirectory() as td:
            spec = os.path.join(td, "spec.bin")
            S.write_spec(spec, sysm, [kp], [psi])
            procs = []
            for w in range(workers):
                b0 = (w * bands_per_worker) % nb
                procs.append(subprocess.Popen([O.REF_BENCH, "time", spec, os.path.join(td, f"wd{w}"), "0", str(b0),
                                               str(bands_per_worker)], stdout=subprocess.PIPE,
                                              stderr=subprocess.DEVNULL, text=True))
            secs = []
            for p in procs:
                out, _ = p.communicate()
                if p.returncode != 0:
                    raise RuntimeError("reference driver failed")
                secs.append(json.loads(out.strip().splitlines()[-1])["seconds"])
        t = max(secs)
        return dict(value=workers * bands_per_worker / t, per_core_value=bands_per_worker / statistics.median(secs),
                    cores=workers, kind="reference", seconds=t, cpu=cpu_model(),
                    sample=f"{workers} single-threaded reference processes (g++ -O3) x {bands_per_worker} bands "
                           f"(npw={kp.npw}), H|psi> time only")
    # fallback: the oracle port, threads over bands
    O.build()
    nbs = min(nb, workers * bands_per_worker)
    t0 = time.perf_counter()
    O.hpsi(sysm, kp, psi[:nbs], threads=workers)
    t = time.perf_counter() - t0
    return dict(value=nbs / t, per_core_value=nbs / t / workers, cores=workers, kind="port", seconds=t,
                cpu=cpu_model(), sample=f"oracle port on {workers} threads x {nbs} bands (npw={kp.npw})")

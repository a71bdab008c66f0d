"""Benchmark: full Debye patterns of the spinel-like 10 nm nanoparticle.

Workload ``spinel_10nm`` (cudebye_gb300.lattice): 117,945 atoms in three
species (6 pair types), histogram bin 1e-3 A over 104,002 bins,
6,001 2theta points (10-130 deg, 0.02 deg, 1.5406 A). One step = one full
pattern: every pair histogram recomputed on the device, then the Debye sum
(tensor-core split contraction). Metric: G binned pairs/s, where binned
pairs = sum_{a<b} n_a n_b + sum_a n_a(n_a+1)/2 (the reference's "Distances
Expected", cuDebye-v15.cu:372,:396) per pattern.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

``value``: device time per step (CUDA events on the engine's launch stream,
model resident in HBM, L2 flushed between steps). ``e2e``: the same metric
through the C ABI with host buffers (upload from host coordinates, pattern,
intensities read back, model freed) per step. ``cpu_baseline``: the oracle
(C/OpenMP) on all host cores over one full pattern. ``--impl reference``
times the reference's arithmetic on the host cores (the C/OpenMP oracle;
the reference program itself has no CPU path), one full pattern per step,
and runs the reference program once on the GPU beside it. Further legs:
``plain_small`` (5,000 atoms), ``batch256`` (the 256-model mix, batched vs
the plain FP32 GPU form), ``precision`` (20,000 q), ``file_io``,
``serving`` (Poisson arrivals of fresh requests); the benchmark spec sums them
up last on the line. Multi-GPU: independent replicas per rank (the path
needs no exchange).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "G binned pairs/s"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
# DRAM bytes per launch of the top kernels, from ncu captures (see the
# summaries beside it); keyed by kernel, then workload.
TRAFFIC_PATH = os.path.join(ROOT, "profiles", "traffic.json")


def measured_traffic(kernel, workload):
    try:
        with open(TRAFFIC_PATH) as f:
            t = json.load(f)
        return t[kernel][workload]["dram_bytes_per_launch"]
    except (OSError, KeyError, ValueError):
        return None


def launches_per_pattern(mode, npairs):
    """Kernels one dbx_pattern call launches on a resident model whose q grid
    is unchanged: the histogram (zero, tiles, reduce), the prefactor (form
    factors, pair products), then for the tensor-core sum the self term,
    weights, contraction and reduce, for the direct sums one launch per 16
    pair types."""
    n = 3 + 2
    if mode == "tc":
        return n + 4
    return n + (npairs + 15) // 16


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0,
                "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.first = 0
        self.last = None

    def start(self, wait_s=5.0):
        """Start sampling before the warm-up, so that nvidia-smi's own
        start-up (driver queries while it initialises) stays out of the timed
        steps, and wait for its first line."""
        import atexit
        self.__enter__()
        atexit.register(self.__exit__)  # the sampler ends with the process
        t0 = time.time()
        while self.proc and not self.lines and time.time() - t0 < wait_s:
            time.sleep(0.01)
        return self

    def mark(self):
        """Start of the timed region: summary() covers the samples from here
        to stop()."""
        self.first = len(self.lines)

    def stop(self):
        self.last = len(self.lines)
        t0 = time.time()  # a short region: wait for the sample just after it
        while (self.proc and len(self.lines) <= max(self.first, self.last)
               and time.time() - t0 < 0.5):
            time.sleep(0.01)
        self.__exit__()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        last = len(self.lines) if self.last is None else self.last
        lines = self.lines[self.first:last]
        where = "during the timed region"
        if not lines:  # a region shorter than the sampling period: the
            # samples on either side of it
            lines = self.lines[max(0, self.first - 1):last + 1]
            where = "the samples just before and after the timed region"
        for l in lines:
            p = [v.strip() for v in l.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm),
                "sampled": where}


def job_times(times, ws, device=None):
    """Whole-job times of one replica per rank: the max over ranks of each
    entry (the slowest replica ends the job)."""
    if ws <= 1:
        return [float(t) for t in times]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in times], dtype=torch.float64,
                     device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


WORKLOADS = {
    # the metric's configuration: ~118k-atom spinel-like 10 nm particle
    "spinel_10nm": lambda L: L.spinel_10nm(),
    # smaller cases of the same kernels, for profiler captures
    "spinel_medium": lambda L: L.spinel(radius=30.0, target=25000, seed=7,
                                        label="spinel_medium"),
    "plain_small": lambda L: L.plain_small(),
}
WORKLOAD = "spinel_10nm"


def workload():
    from cudebye_gb300 import lattice
    return WORKLOADS[WORKLOAD](lattice)


def cpu_model():
    """The host CPU's model name (lscpu "Model name", else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True,
                             timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def oracle_pattern(m, K, threads=0):
    """One full pattern by the oracle on the host cores (C/OpenMP): every
    pair histogram of every atom (cuDebye-v15.cu:88-146) and the FP64 Debye
    sum at every q (:493-538). Returns (seconds, histogram seconds)."""
    from oracle import pyoracle as orc
    orc.lib()
    t0 = time.perf_counter()
    hists, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins,
                                      threads)
    t1 = time.perf_counter()
    orc.intensity(K, hists, m.species, m.rstep, threads=threads)
    t2 = time.perf_counter()
    if bad:
        raise RuntimeError("oracle: %d distances beyond rmax" % bad)
    return t2 - t0, t1 - t0


def cpu_baseline(m, K, threads=0):
    """The oracle timed on one full pattern of the workload (no sampling,
    no extrapolation) on all host cores."""
    t, th = oracle_pattern(m, K, threads)
    cores = threads or os.cpu_count()
    return {"value": m.pairs / t / 1e9, "unit": METRIC, "cores": cores,
            "cpu_model": cpu_model(), "kind": "port",
            "sample": "one full pattern of %s: oracle (C/OpenMP, %d threads), "
                      "all %d pair histograms (%.2f s) + FP64 Debye sum at all "
                      "%d q (%.2f s)" % (m.label, cores, len(m.counts) *
                                         (len(m.counts) + 1) // 2, th,
                                         len(K), t - th),
            "pattern_s": t}


def batch_bench(eng, steps=5, seed=3, nmodels=256, plain_models=None):
    """The batched form: 256 independent models (sc / fcc / spinel-like,
    N log-uniform 2k-60k, 1-4 species, sigma U[0.03,0.1], B U[0.2,1.5]) on
    the 6,001-point q grid. Patterns/s of (a) the batched engine (one
    histogram launch + one tensor-core contraction for all 256 models,
    CUDA-graph replay) and (b) the plain unbatched FP32 GPU form (model by
    model: one-thread-per-pair global-atomic histogram + FP32 direct Debye
    sum). Max relative error of every pattern of (a) against the FP64
    direct sum (every 10th q): the reference's arithmetic on the device,
    which the tests hold within 1e-11 of the CPU FP64 oracle."""
    from cudebye_gb300 import lattice
    mods = lattice.batch256(seed=seed, nmodels=nmodels)
    tt, K = mods[0].k_grid()
    sp = [s for m in mods for s in m.species]
    nb = [m.nbins for m in mods]
    hs = [eng.upload(m.xyz, m.counts) for m in mods]
    pairs = sum(m.pairs for m in mods)
    try:
        I = eng.patterns(hs, 1e-3, nb, sp, K)  # plan, autotune, graph capture
        I = eng.patterns(hs, 1e-3, nb, sp, K)
        ts = []
        for _ in range(steps):
            t0 = time.perf_counter()
            I = eng.patterns(hs, 1e-3, nb, sp, K)
            ts.append(time.perf_counter() - t0)
        t_tc = float(np.median(ts))
        # every pattern's max relative error at every 10th q against the
        # FP64 direct sum of its resident histograms (dbx_pattern_errors)
        per = eng.pattern_errors(hs, 1e-3, nb, sp, K, I, q_stride=10).tolist()
        worst = max(per)
        # the plain form over the whole mix (a smaller count only for quick
        # runs: every `step`-th model, scaled per pattern)
        step = 1 if not plain_models else max(1, len(mods) // plain_models)
        sub = list(range(0, len(mods), step))
        sp_sub = [s for i in sub for s in mods[i].species]
        t0 = time.perf_counter()
        eng.patterns([hs[i] for i in sub], 1e-3, [nb[i] for i in sub], sp_sub,
                     K, mode="plain")
        t_plain = (time.perf_counter() - t0) * len(mods) / len(sub)
    finally:
        for h in hs:
            h.free()
    return {
        "models": len(mods), "binned_pairs": int(pairs),
        "atoms_total": int(sum(m.natoms for m in mods)),
        "patterns_per_s_batched": len(mods) / t_tc,
        "patterns_per_s_plain": len(mods) / t_plain,
        "speedup_batched_vs_plain": t_plain / t_tc,
        "ms_per_batch": t_tc * 1e3,
        "max_rel_err_vs_fp64": worst, "err_models_checked": len(per),
        "median_pattern_max_rel_err": float(np.median(per)),
        "patterns_over_1e-6": int(sum(e > 1e-6 for e in per)),
        "err_reference": "FP64 direct sum on the device (every 10th q), the "
                         "reference's arithmetic; tests hold it within 1e-11 "
                         "of the CPU FP64 oracle",
        "timing": "host wall clock around dbx_patterns (H2D species/K, graph "
                  "replay, D2H of all intensities), median of %d passes; "
                  "plain form: one pass over %d of %d models"
                  % (steps, len(sub), len(mods)),
    }


def precision_bench(eng, reps=3):
    """The precision form: the spinel model's histograms (resident) summed
    on the 20,000-point q grid (2theta 5-150 deg at 0.7107 A) by the exact
    tensor-core split, the three-product BF16x3 and TF32-split forms, the
    plain FP32 direct sum and the FP64 direct sum (the reference's
    arithmetic, the error reference). Per form: device time of the Debye sum (CUDA events,
    median of `reps`) and max relative error over all q."""
    from cudebye_gb300 import lattice
    m = lattice.precision()
    tt, K = m.k_grid()
    mod = eng.upload(m.xyz, m.counts)
    res = {}
    try:
        eng.histogram(mod, m.rstep, m.nbins)
        outs = {}
        for mode in ("fp64", "tc", "tc3", "tf32", "fp32"):
            ts, ws = [], []
            for _ in range(reps + 1):
                t0 = time.perf_counter()
                outs[mode] = eng.intensity(mod, m.rstep, m.nbins, m.species, K,
                                           mode=mode)
                ws.append(time.perf_counter() - t0)
                ts.append(eng.timing()["debye"])
            res[mode] = {"debye_kernel_ms": float(np.median(ts[1:])),
                         "call_ms": float(np.median(ws[1:])) * 1e3}
        ref = outs["fp64"]
        for mode in ("tc", "tc3", "tf32", "fp32"):
            rel = np.abs(outs[mode] - ref) / np.abs(ref)
            res[mode]["max_rel_err"] = float(np.max(rel))
            res[mode]["median_rel_err"] = float(np.median(rel))
    finally:
        mod.free()
    return {"workload": "spinel_10nm histograms, %d q (2theta 5-150, "
                        "0.7107 A)" % len(K),
            "bins": m.nbins, "pair_types": len(m.counts) * (len(m.counts) + 1) // 2,
            "error_reference": "fp64 direct sum (device)",
            "timing": "debye_kernel_ms: CUDA events around the contraction "
                      "kernel (tc, tc3, tf32) or the direct-sum kernel; call_ms: "
                      "host wall clock of dbx_intensity on resident "
                      "histograms (prefactors, weights, reduction, D2H)",
            "forms": {"tc": "exact 4-digit bf16 split (10 products)",
                      "tc3": "BF16x3: 2 digits, 3 products",
                      "tf32": "TF32-split: tf32 hi/lo parts, 3 products, FP32 "
                              "accumulation per 256-bin chunk, FP64 chunk sums",
                      "fp32": "FP32 direct sum", "fp64": "FP64 direct sum"},
            "results": res}


def io_bench(eng, nfiles=16, seed=8):
    """The file surface: (a) the reference's shipped Gamma-Al2O3 input
    (117,936 atoms, rstep 1e-4, hist 2: six .debx files and the .debI) run
    by the command line from its text and its binary form, and in-process
    (dbx_run_deb, context already open); the reference logged 2.191 s to
    load this file and 11.563 s for histograms, checks, .debx writing and
    the Debye sum on a GTX 980 Ti (Data/cmd-logfile.txt:94, :500-501).
    (b) A directory of `nfiles` small models (2k-20k atoms, hist 0): the
    directory driver (dbx_run_dir, batched) against one command-line
    process per file, which is how the reference's multisim runs them."""
    import lzma
    import shutil
    import subprocess
    import tempfile
    import cudebye_gb300 as cd
    from cudebye_gb300 import lattice
    out = {}
    tmp = tempfile.mkdtemp(prefix="dbx_io_")
    try:
        src = os.path.join(tmp, "Gamma.deb")
        with open(os.path.join(ROOT, "tests", "golden",
                               "GammaAl2O3_10nm.deb.xz"), "rb") as f:
            raw = lzma.decompress(f.read())
        with open(src, "wb") as f:
            f.write(raw)
        t0 = time.perf_counter()
        cd.deb_pack(src, os.path.join(tmp, "Gamma.debb"))
        out["pack_s"] = time.perf_counter() - t0
        for form, path in (("text", src), ("binary", os.path.join(tmp, "Gamma.debb"))):
            ts = []
            for _ in range(2):
                t0 = time.perf_counter()
                r = subprocess.run([cd.CLI_PATH, path, "--out",
                                    os.path.join(tmp, "o_" + form), "--quiet"],
                                   capture_output=True, text=True)
                ts.append(time.perf_counter() - t0)
                if r.returncode != 0:
                    raise RuntimeError(r.stderr)
            out["cli_gamma_%s_s" % form] = min(ts)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            eng.run_deb(src, os.path.join(tmp, "o_inproc"))
            ts.append(time.perf_counter() - t0)
        out["run_deb_gamma_s"] = min(ts)
        out["reference_logged_gamma_s"] = {"load": 2.191, "compute_and_write": 11.563,
                                           "gpu": "GTX 980 Ti"}
        # device phases of the Gamma pattern (3.56 M bins of 1e-4 A: the
        # histogram in 31 shared-memory windows), CUDA events, median of 3
        d = cd.read_deb(src)
        _, Kg = cd.k_grid(d.lam, d.tt_min, d.tt_max, d.tt_step)
        nbg = cd.channels(d.rmax, d.rstep)
        mg = eng.upload(d.xyz, d.counts)
        try:
            ph = []
            for _ in range(4):
                eng.pattern(mg, d.rstep, nbg, d.species, Kg)
                ph.append(eng.timing())
        finally:
            mg.free()
        out["gamma_device_ms"] = {k: float(np.median([t[k] for t in ph[1:]]))
                                  for k in ("hist", "hist_reduce", "debye")}
        d = os.path.join(tmp, "dir")
        os.mkdir(d)
        rng = np.random.default_rng(seed)
        for i in range(nfiles):
            lattice.random_model(rng, 2000, 20000, lattice.GRID_CU, "f%d" % i,
                                 seed).write_deb(os.path.join(d, "f%02d.deb" % i))
        t0 = time.perf_counter()
        eng.run_dir(d)
        out["dir_driver_s"] = time.perf_counter() - t0
        for f in os.listdir(d):
            if f.endswith("I"):
                os.remove(os.path.join(d, f))
        t0 = time.perf_counter()
        for f in sorted(os.listdir(d)):
            r = subprocess.run([cd.CLI_PATH, os.path.join(d, f), "--quiet"],
                               capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(r.stderr)
        out["cli_per_file_s"] = time.perf_counter() - t0
        out["files"] = nfiles
        out["dir_speedup"] = out["cli_per_file_s"] / out["dir_driver_s"]
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return out


class RequestFeed:
    """Fresh serving requests from spawned worker processes
    (lattice.request_worker): each request has its own geometry and its own
    2theta grid, made off the submitting thread so that the arrival
    schedule is kept."""

    def __init__(self, seed, workers=None):
        import multiprocessing as mp
        from cudebye_gb300 import lattice
        self.lattice = lattice
        n = workers or max(2, min(6, (os.cpu_count() or 4) // 2))
        ctx = mp.get_context("spawn")
        self.q = ctx.Queue(maxsize=256)
        self.stop_ev = ctx.Event()
        self.procs = [ctx.Process(target=lattice.request_worker,
                                  args=(seed * 1000 + i, self.q, self.stop_ev),
                                  daemon=True) for i in range(n)]
        for p in self.procs:
            p.start()
        self.waited_s = 0.0  # time the arrival loop waited for a request

    def get(self):
        import queue
        t0 = time.perf_counter()
        while True:
            try:
                item = self.q.get(timeout=5.0)
                break
            except queue.Empty:
                if not any(p.is_alive() for p in self.procs):
                    raise RuntimeError("request workers exited")
        self.waited_s += time.perf_counter() - t0
        return self.lattice.model_from_item(item)

    def close(self):
        import queue
        self.stop_ev.set()
        t0 = time.perf_counter()
        while any(p.is_alive() for p in self.procs) and time.perf_counter() - t0 < 20:
            try:
                while True:
                    self.q.get_nowait()
            except queue.Empty:
                pass
            for p in self.procs:
                p.join(timeout=0.05)
        for p in self.procs:
            if p.is_alive():
                p.terminate()


def serving_bench(rates=(5, 20, 50, 100, 200, 400, 800), seconds=6.0, seed=4,
                  budget_gib=16):
    """The serving form: Poisson arrivals at each rate for `seconds`; each
    new request is a fresh spherical lattice model of 1,000-200,000 atoms
    (log-uniform, 1-4 species, random orientation and jitter) with its own
    2theta grid of 2,000-20,000 points, or, with probability 0.2, a
    re-scoring of one of the 64 models completed last with new B factors. Latency = submit to
    result, measured by the server. The server admits by HBM footprint
    within `budget_gib`, evicting idle resident models; a re-score of a
    model evicted meanwhile fails with DBX_ERR_MODEL and is counted, not
    timed."""
    import collections
    import concurrent.futures as cf
    import cudebye_gb300 as cd
    from cudebye_gb300 import lattice
    rng = np.random.default_rng(seed)
    feed = RequestFeed(seed)
    out = []
    try:
        with cd.Server(0, hbm_budget=budget_gib << 30) as srv:
            for _ in range(4):  # warm-up
                m = feed.get()
                K = m.k_grid()[1]
                srv.wait(srv.submit(m.species, m.rstep, m.nbins, K, xyz=m.xyz,
                                    counts=m.counts), len(K))
            for rate in rates:
                # re-scores go to one of the 64 models completed last (a
                # client re-scores what it has just seen; older ones may
                # have been evicted under the HBM budget)
                lat, done_t, failed = [], [], []
                resident = collections.deque(maxlen=64)
                lock = threading.Lock()
                ex = cf.ThreadPoolExecutor(max_workers=64)
                atoms = []

                def waiter(t, nq, rec, t0):
                    try:
                        I, mid, ms = srv.wait(t, nq)
                    except cd.DebyeError as err:  # re-score of an evicted model
                        with lock:
                            failed.append(err.code)
                        return
                    with lock:
                        lat.append(ms)
                        done_t.append(time.perf_counter() - t0)
                        if rec is not None:
                            resident.append((mid,) + rec)

                waited0 = feed.waited_s
                t0 = time.perf_counter()
                tnext, futs, nsub, nres, late = 0.0, [], 0, 0, 0.0
                while tnext < seconds:
                    with lock:
                        can = bool(resident)
                    if can and rng.random() < 0.2:
                        with lock:
                            mid, names, rstep, nbins, K = resident[
                                int(rng.integers(len(resident)))]
                        sp = [lattice.species(n, 1.0, float(rng.uniform(0.2, 1.5)))
                              for n in names]
                        req = (sp, rstep, nbins, K, dict(model=mid), None)
                    else:
                        m = feed.get()
                        K = m.k_grid()[1]
                        req = (m.species, m.rstep, m.nbins, K,
                               dict(xyz=m.xyz, counts=m.counts),
                               (m.names, m.rstep, m.nbins, K))
                        atoms.append(m.natoms)
                    now = time.perf_counter() - t0
                    if now < tnext:
                        time.sleep(tnext - now)
                    else:
                        late = max(late, now - tnext)
                    sp, rstep, nbins, K, kw, rec = req
                    t = srv.submit(sp, rstep, nbins, K, **kw)
                    futs.append(ex.submit(waiter, t, len(K), rec, t0))
                    if rec is None:
                        nres += 1
                    nsub += 1
                    tnext += rng.exponential(1.0 / rate)
                for f in futs:
                    f.result()
                ex.shutdown()
                span = max(done_t) if done_t else seconds
                out.append({"rate": rate, "submitted": nsub, "rescored": nres,
                            "failed_evicted": len(failed),
                            "patterns_per_s": len(lat) / span,
                            "completed": len(lat),
                            "p50_ms": float(np.percentile(lat, 50)),
                            "p90_ms": float(np.percentile(lat, 90)),
                            "p99_ms": float(np.percentile(lat, 99)),
                            "p999_ms": float(np.percentile(lat, 99.9)),
                            "max_ms": float(np.max(lat)),
                            "mean_atoms": float(np.mean(atoms)) if atoms else 0.0,
                            "max_arrival_lag_s": late,
                            "feed_wait_s": feed.waited_s - waited0})
            st = srv.stats()
    finally:
        feed.close()
    sat = max([o["rate"] for o in out
               if o["patterns_per_s"] >= 0.9 * o["rate"]] or [0])
    return {"rates": out, "saturation_req_per_s": sat,
            "seconds_per_rate": seconds,
            "requests": "fresh geometry and 2theta grid per new request "
                        "(lattice.RequestStream in %d spawned workers)"
                        % len(feed.procs),
            "hbm_budget_gib": budget_gib,
            "rounds": st["rounds"], "evictions": st["evictions"],
            "timing": "host clock; latency measured by the server from "
                      "submit to result (incl. upload, queueing, readback)"}


def reference_program(m, block=16, grid=4096, timeout=900):
    """The reference's own CUDA program (cuDebye-v15.cu, built from an
    edited copy by `make -C oracle ref`: CUDA 13 / gcc fixes, --fmad=false)
    run once on this workload as a GPU timing beside the CPU arm. The
    workload is written as a .deb with hist 0 (intensities only, so no
    .debx writing inside its compute phase) and the launch grid `block`,
    `grid` of its line 1. Reported: the process wall time and the phases the
    program prints itself (cuDebye-v15.cu:840, :922, :971; clock(), i.e.
    process CPU time, which its synchronous spin waits keep close to wall
    time)."""
    import re
    import shutil
    import tempfile
    from oracle import pyoracle
    if not os.path.exists(pyoracle.REF_BIN):
        return {"unavailable": "reference program not built (its source "
                               "copy was never made here)"}
    tmp = tempfile.mkdtemp(prefix="dbx_refprog_")
    try:
        deb = os.path.join(tmp, "w.deb")
        m.write_deb(deb, block=block, grid=grid, hist=0)
        t0 = time.perf_counter()
        r = subprocess.run([pyoracle.REF_BIN, deb], capture_output=True,
                           encoding="latin-1", timeout=timeout)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            return {"unavailable": "reference program exit %d: %s"
                    % (r.returncode, (r.stdout + r.stderr)[-300:])}

        def phase(label):
            g = re.search(label + r"\s*([0-9.eE+-]+) s", r.stdout)
            return float(g.group(1)) if g else None
        load = phase(r"Time for Loading the Input File:")
        alloc = phase(r"Time for Allocating the necessary Memory on the Device:")
        calc = phase(r"Evaluation of the Debye Double Sum:")
        I = np.loadtxt(deb + "I")[:, 1]
        return {"program": "cuDebye-v15.cu, CUDA 13 edits, nvcc --fmad=false, sm_103a",
                "deb_line1": "0 %d %d" % (block, grid), "hist": 0,
                "wall_s": wall, "load_s": load, "alloc_s": alloc,
                "compute_s": calc,
                "value": m.pairs / calc / 1e9 if calc else None,
                "unit": METRIC,
                "warnings": r.stdout.count("WARNING"),
                "intensity_sum": float(np.sum(I))}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def reference_program_batch(step=16, seed=3):
    """The reference program on every `step`-th model of the 256-model mix,
    one process per model (how the reference's multisim runs a folder of
    models), as a GPU timing beside the batched engine: patterns/s over the
    program's own compute phases and over the processes' wall time."""
    from cudebye_gb300 import lattice
    models = lattice.batch256(seed=seed)[::step]
    runs = []
    for m in models:
        r = reference_program(m)
        if "unavailable" in r:
            return r
        runs.append(r)
    comp = sum(r["compute_s"] for r in runs)
    wall = sum(r["wall_s"] for r in runs)
    return {"models": len(runs),
            "sample": "every %dth model of the 256-model mix (seed %d), "
                      "hist 0, line 1 '0 16 4096'" % (step, seed),
            "binned_pairs": int(sum(m.pairs for m in models)),
            "compute_s": comp, "wall_s": wall,
            "patterns_per_s_compute": len(runs) / comp,
            "patterns_per_s_process": len(runs) / wall}


def run_config(m, K):
    """The `config` of both arms' lines (the same keys and values)."""
    return {"workload": m.label, "atoms": m.natoms,
            "species": len(m.counts),
            "pair_types": len(m.counts) * (len(m.counts) + 1) // 2,
            "bins": m.nbins, "rstep": m.rstep, "q_points": len(K),
            "binned_pairs": m.pairs,
            "l2": "engine arm: L2 flushed between steps (256 MB write); "
                  "reference arm: host caches not flushed"}


def run_reference(args):
    """The reference arm: the reference's arithmetic (the C/OpenMP oracle;
    the reference program has no CPU path) on all host cores, one full
    pattern per step: every pair histogram and the FP64 Debye sum at every
    q. Rank 0 only."""
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    m = workload()
    tt, K = m.k_grid()
    for _ in range(args.warmup):  # untimed: page faults, thread start-up
        oracle_pattern(m, K)
    ts, th = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t, h = oracle_pattern(m, K)
        ts.append(t)
        th.append(h)
    wall = time.perf_counter() - t0
    t_step = float(np.mean(ts))
    v = m.pairs / t_step / 1e9
    cores = os.cpu_count()
    line = {
        "metric": METRIC, "value": v, "unit": METRIC, "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded spinel-like nanoparticle)",
        "config": run_config(m, K),
        "debye_mode": "fp64",
        "parallelism": "%d host threads of rank 0" % cores,
        "cpu_baseline": {"value": v, "unit": METRIC, "cores": cores,
                         "cpu_model": cpu_model(), "kind": "port",
                         "sample": "every step one full pattern (no sampling): "
                                   "oracle histograms %.2f s + FP64 Debye sum "
                                   "%.2f s (means)" % (np.mean(th),
                                                       t_step - np.mean(th))},
        "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "timed_region_s": wall,
    }
    if not args.no_refprog:
        line["reference_program_gpu"] = reference_program(m)
        line["reference_program_gpu_batch256"] = reference_program_batch()
    print(json.dumps(line))
    return 0


def pattern_leg(eng, stream, m, K, mode, steps, warmup, flush, clk=None,
                barrier=None):
    """Full patterns of one resident model: `steps` device-timed passes (CUDA
    events on the engine's stream, L2 flushed by `flush` before each), then
    `steps` end-to-end passes through the C ABI from host coordinates
    (upload incl. sort and plan, pattern, intensities read back, model
    freed). The histogram total is checked against the pair count."""
    import torch
    import cudebye_gb300 as cd
    eng.set_stream(stream.cuda_stream)
    model = eng.upload(m.xyz, m.counts)
    out = np.zeros(len(K))
    try:
        for _ in range(warmup):
            eng.pattern(model, m.rstep, m.nbins, m.species, K, mode=mode, out=out)
        h = eng.histogram(model, m.rstep, m.nbins)
        assert int(h.sum()) == m.pairs, "histogram total != binned pairs"
        phase = {k: [] for k in cd.TIMERS}
        ev = [(torch.cuda.Event(enable_timing=True),
               torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        if barrier:
            barrier()
        torch.cuda.synchronize()
        if clk:
            clk.mark()
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()  # L2 flush (256 MB > 129 MB L2), not timed
            ev[i][0].record(stream)
            eng.pattern(model, m.rstep, m.nbins, m.species, K, mode=mode, out=out)
            ev[i][1].record(stream)
            for k, v in eng.timing().items():
                phase[k].append(v)
        if barrier:
            barrier()
        torch.cuda.synchronize()
        h2d0, d2h0 = eng.traffic()
        eng.set_stream(None)
        e2e_s = []
        for i in range(steps):
            t0 = time.perf_counter()
            mod2 = eng.upload(m.xyz, m.counts)
            eng.pattern(mod2, m.rstep, m.nbins, m.species, K, mode=mode, out=out)
            mod2.free()
            e2e_s.append(time.perf_counter() - t0)
        h2d1, d2h1 = eng.traffic()
        if clk:
            clk.stop()
        torch.cuda.synchronize()
    finally:
        model.free()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    return {"t_step": float(np.mean(step_ms)) / 1e3,
            "t_e2e": float(np.mean(e2e_s)),
            "phase_ms": {k: float(np.mean(v)) for k, v in phase.items()},
            "h2d": (h2d1 - h2d0) // steps, "d2h": (d2h1 - d2h0) // steps}


def sig(v, n=4):
    """v rounded to n significant digits (compact summary values)."""
    return float("%.*g" % (n, v)) if isinstance(v, float) else v


def run_engine(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from cudebye_gb300 import build as cbuild
    cbuild.build()
    import cudebye_gb300 as cd

    m = workload()
    tt, K = m.k_grid()
    eng = cd.Engine(local)
    stream = torch.cuda.Stream(device=local)
    eng.set_timing(True)
    mode = args.mode
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=local)
    clk = Clocks(local).start()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    lead = pattern_leg(eng, stream, m, K, mode, args.steps, args.warmup, flush,
                       clk=clk, barrier=barrier)
    t_step, t_e2e = job_times([lead["t_step"], lead["t_e2e"]], ws, device=local)
    if rank != 0:
        eng.close()
        return 0
    pk, pk_kind = peaks()
    clocks = clk.summary()
    ph = lead["phase_ms"]
    npair_types = len(m.counts) * (len(m.counts) + 1) // 2
    total_pairs = m.pairs * ws
    value = total_pairs / t_step / 1e9
    # roofline of the dominant kernel (the histogram), and of the
    # tensor-core contraction beside it
    sm_mhz = clocks["sm_mhz"] or pk.get("sm_max_mhz", 2070.0)
    # FP32-pipe bound of the reference's exact bin formula: 16 FP32
    # operations per pair (3 sub, 3 mul, 2 add, square root as estimate + 4
    # correction ops, 1 mul, 2 for roundf), SMs x 128 FP32 lanes per clock.
    # Packed FP32x2 instructions do two of these per lane and issue slot, so
    # a kernel can exceed this bound. (The tile kernels do roundf with one
    # FP32 add and two integer operations; the bound keeps the formula's 16.)
    ops = 16
    peak = nsm * 128 * sm_mhz * 1e6 / ops / 1e9
    ach = m.pairs / (ph["hist"] / 1e3) / 1e9
    roof = {"kernel": "hist_tiles_kernel", "bound": "alu",
            "achieved": ach, "peak": peak, "unit": "Gpair/s",
            "frac": ach / peak,
            "traffic": measured_traffic("hist_tiles_kernel", m.label),
            "traffic_unit": "DRAM bytes per launch (ncu)",
            "algorithmic_bytes": 16 * m.natoms + 8 * m.nbins * npair_types,
            "peak_basis": "FP32 pipe, %d ops/pair, %d SMs at %.0f MHz (median "
                          "sampled SM clock)" % (ops, nsm, sm_mhz)}
    # the same launch against the measured HBM copy bandwidth: the kernel
    # moves O(atoms + bins) bytes for O(atoms^2) work, so it is far from it
    alg_gbs = roof["algorithmic_bytes"] / (ph["hist"] / 1e3) / 1e9
    roof["hbm_view"] = {"achieved": alg_gbs, "peak": pk["hbm_gbs"],
                        "unit": "GB/s", "frac": alg_gbs / pk["hbm_gbs"],
                        "peak_basis": "hbm_gbs, %s" % pk_kind}
    flops = 2.0 * len(K) * m.nbins * npair_types
    tc_ach = flops / (ph["debye"] / 1e3) / 1e12
    # bf16 MMA work the split form issues: per 128-row x 64-chunk x 256-bin
    # tile, 10 digit-pair products of 2 x 128 x 64 x 256 FLOP (four MMAs of
    # N = 256, 192, 128, 64 per K step)
    qp = (len(K) + 127) // 128 * 128
    nch = (m.nbins + 255) // 256  # 256-bin chunks per pair type
    col_tiles = npair_types * ((nch + 63) // 64)
    issued = (2 * qp // 128) * col_tiles * 10 * 2.0 * 128 * 64 * 256
    issued_tf = issued / (ph["debye"] / 1e3) / 1e12
    roof_tc = {"kernel": "gemm_persistent_kernel", "bound": "tensor",
               "achieved": tc_ach, "peak": pk["bf16_tflops"],
               "unit": "TFLOP/s", "frac": tc_ach / pk["bf16_tflops"],
               "traffic": measured_traffic("gemm_persistent_kernel", m.label),
               "flops_basis": "2 x q x bins x pair types (one FP64-exact "
                              "sinc product per count); the split form "
                              "issues 10 bf16 MMAs per product",
               "peak_basis": "bf16 dense, %s" % pk_kind,
               "issued": {"achieved": issued_tf, "frac": issued_tf / pk["bf16_tflops"],
                          "unit": "TFLOP/s",
                          "basis": "bf16 MMA FLOP issued: 10 digit-pair products "
                                   "per 128 x 64 x 256 tile (MMAs of N = 256, "
                                   "192, 128, 64 per K step), %d tiles" %
                                   ((2 * qp // 128) * col_tiles)}}
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded spinel-like nanoparticle)",
        "config": run_config(m, K),
        "debye_mode": mode,
        "parallelism": "replicas" if ws > 1 else "single",
        "patterns_per_s": ws / t_step,
        "phase_ms": ph,
        "e2e": {"value": total_pairs / t_e2e / 1e9, "unit": METRIC,
                "h2d_bytes_per_step": lead["h2d"],
                "d2h_bytes_per_step": lead["d2h"],
                "ms_per_step": t_e2e * 1e3},
        "gpu_launches": args.steps * launches_per_pattern(mode, npair_types),
        "roofline": roof,
        "roofline_debye": roof_tc,
        "clocks": clocks,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = {k: v for k, v in cpu_baseline(m, K).items()
                                if k != "pattern_s"}
    if not args.no_small:  # the small-input regime: plain_small, 5,000 atoms
        from cudebye_gb300 import lattice
        ms = WORKLOADS["plain_small"](lattice)
        _, Ks = ms.k_grid()
        leg = pattern_leg(eng, stream, ms, Ks, mode, args.steps, args.warmup,
                          flush)
        small = {"config": run_config(ms, Ks),
                 "value": ms.pairs / leg["t_step"] / 1e9, "unit": METRIC,
                 "ms_per_step": leg["t_step"] * 1e3,
                 "patterns_per_s": 1.0 / leg["t_step"],
                 "phase_ms": leg["phase_ms"],
                 "e2e": {"value": ms.pairs / leg["t_e2e"] / 1e9, "unit": METRIC,
                         "h2d_bytes_per_step": leg["h2d"],
                         "d2h_bytes_per_step": leg["d2h"],
                         "ms_per_step": leg["t_e2e"] * 1e3}}
        if not args.no_cpu:
            small["cpu_baseline"] = {k: v for k, v in cpu_baseline(ms, Ks).items()
                                     if k != "pattern_s"}
        line["plain_small"] = small
    if not args.no_batch:
        line["batch256"] = batch_bench(eng, plain_models=args.plain_models)
    if not args.no_io:
        line["file_io"] = io_bench(eng)
    if not args.no_precision:
        line["precision"] = precision_bench(eng)
    eng.close()
    if not args.no_serve:
        rates = [int(r) for r in args.serve_rates.split(",")]
        line["serving"] = serving_bench(rates=rates, seconds=args.serve_seconds)
    # The benchmark spec's figures, last on the line: batched vs plain patterns/s
    # on the 256-model mix with the worst error, p50/p99 under the serving
    # load, and the small-input leg.
    ns = {}
    if "batch256" in line:
        b = line["batch256"]
        ns["batch256"] = {k: sig(b[k]) for k in (
            "patterns_per_s_batched", "patterns_per_s_plain",
            "speedup_batched_vs_plain", "max_rel_err_vs_fp64",
            "patterns_over_1e-6", "err_models_checked")}
    if "serving" in line:
        r = [o for o in line["serving"]["rates"] if o["rate"] == 200] or \
            line["serving"]["rates"][-1:]
        if r:
            ns["serving"] = {k: sig(r[0][k]) for k in (
                "rate", "submitted", "patterns_per_s", "p50_ms", "p99_ms")}
            ns["serving"]["saturation_req_per_s"] = \
                line["serving"]["saturation_req_per_s"]
    if "precision" in line:
        r = line["precision"]["results"]
        ns["precision_20000q_max_rel_err"] = {
            k: sig(r[k]["max_rel_err"], 2) for k in ("tc", "tf32", "tc3", "fp32")}
    if "file_io" in line and "gamma_device_ms" in line["file_io"]:
        ns["gamma_sample_device_ms"] = {
            k: sig(v, 3) for k, v in line["file_io"]["gamma_device_ms"].items()}
    if "plain_small" in line:
        ns["plain_small"] = {"value": sig(line["plain_small"]["value"]),
                             "e2e": sig(line["plain_small"]["e2e"]["value"])}
    ns["headline"] = {"value": sig(value), "e2e": sig(line["e2e"]["value"]),
                      "hist_frac": sig(roof["frac"], 3)}
    line["north_star"] = ns
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--mode", default="tc", choices=["tc", "fp64", "fp32"])
    ap.add_argument("--no-cpu", action="store_true",
                    help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--workload", default="spinel_10nm",
                    choices=sorted(WORKLOADS))
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the 256-model batched comparison")
    ap.add_argument("--plain-models", type=int, default=0,
                    help="models of the batch timed in the plain form "
                         "(0: all)")
    ap.add_argument("--no-small", action="store_true",
                    help="skip the plain_small (5,000 atoms) leg")
    ap.add_argument("--serve-rates", default="5,20,50,100,200,400,800",
                    help="arrival rates of the serving run (req/s)")
    ap.add_argument("--no-serve", action="store_true",
                    help="skip the serving run")
    ap.add_argument("--no-io", action="store_true",
                    help="skip the file-surface timings")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the 20,000-point precision comparison")
    ap.add_argument("--no-refprog", action="store_true",
                    help="reference arm: skip the reference's own CUDA "
                         "program run")
    ap.add_argument("--serve-seconds", type=float, default=6.0,
                    help="seconds of Poisson arrivals per rate")
    args = ap.parse_args()
    global WORKLOAD
    WORKLOAD = args.workload
    if args.impl == "reference":
        return run_reference(args)
    return run_engine(args)


if __name__ == "__main__":
    sys.exit(main())

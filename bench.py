"""Benchmark of the GB300 spectral-element time step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload batch_shots|sh_rupture|plain_psv|psv_rsf|...]

The default workload is the batched-shot configuration: 256 independent
P-SV problems of uneven size (64^2..512^2 elements, NGLL=5, layered media,
423 M GLL nodes in all, FP32 fields), one launch per time step for the whole
batch, 3000 time steps.  The K benchmark steps are K consecutive parts of
one complete 3000-step solve of every shot from rest, so the timed region is
the whole solve; the W warm-up steps run before it on the same batch, which
is then reset.  The metric is GLL node-steps per second.

For the other workloads a benchmark step is one complete solve of the
workload (all its time steps, fields reset and a 512 MB buffer written
before it).

Reported on one JSON line (rank 0):
  value      node-steps/s of the timed solve, device-timed with CUDA events
             on the solver's own stream, inputs resident on the device
  e2e        the same metric through the C-ABI from host arrays: the
             uploads of every problem, one complete solve, the seismograms
             (and fault series) back to the host, destroy
  roofline   the bulk kernel: algorithmic bytes per launch / average launch
             duration (CUDA events around every launch)
  cpu_baseline  the FP64 oracle (CPU restatement of the reference path) on
             a bounded sample of the same workload; for the batch, the
             smallest shots run to the end, one per host thread, and the
             GPU seismograms of those shots are compared with it
  fp64_plain the FP64 GPU path on the plain P-SV box (batch workload)

--impl reference times the CPU restatement of the reference path (the
reference itself is Fortran and cannot be built here) on the same workload,
set up by the oracle's own restated init.  Under torchrun every rank runs
its own replica (no data exchange); rank 0 prints the line and `value` is
the sum over ranks of work / the slowest rank.
"""
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

BYTES_PER_NODE_STEP = {  # algorithmic bytes per GLL node-step
    # read+write displacement and velocity (ndof words each), read inverse
    # mass (1 word), read the elastic moduli (SH: mu; P-SV: lambda, mu)
    (1, "f32"): 4 * (2 + 2 + 1 + 1),
    (2, "f32"): 4 * (4 + 4 + 1 + 2),
    (1, "f64"): 8 * (2 + 2 + 1 + 1),
    (2, "f64"): 8 * (4 + 4 + 1 + 2),
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="batch_shots",
                   choices=["sh_rupture", "plain_psv", "psv_rsf", "batch_shots", "gradient_shots", "tpv3_inplane"])
    p.add_argument("--nsim", type=int, default=256, help="problems of the batch_shots workload")
    p.add_argument("--scale", type=float, default=1.0)
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64-plain", action="store_true")
    p.add_argument("--time-steps", type=int, default=0,
                   help="time steps per solve (default: all of the workload)")
    return p.parse_args()


class OracleGrid:
    """The mesh and spectral grid from the oracle's restated setup, with the
    Grid methods the workload builders use (so that the reference arm loads
    no product library)."""

    def __init__(self, deck):
        from oracle import pyoracle as po
        self.deck = deck
        self.S = po.OracleSetup(deck, grid_only=True)

    def coord(self):
        return self.S.coord()

    def ibool(self):
        return self.S.ibool()

    def fault_nodes(self, tags=None):
        t1, t2 = tags or (self.deck.fault.tags if self.deck.fault else (5, 6))
        n1 = self.S.boundary(t1)
        if t2 <= 0:
            return n1, None
        n2 = self.S.boundary(t2)
        keep = n1 != n2
        return n1[keep], n2[keep]


def workload_deck(args, grid_cls=None):
    """(deck or (deck, grid), name) of a single-problem workload; grid_cls builds the grid
    the builders evaluate their distributions on (the product's Grid by
    default)."""
    from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, workloads
    prec = PRECISION_MIXED if args.precision == "mixed" else PRECISION_FP64
    kw = {"grid_cls": grid_cls} if grid_cls else {}
    if args.workload == "sh_rupture":
        pair = workloads.sh_rupture(scale=args.scale, precision=prec, **kw)
        name = "SH antiplane rupture, SWF, 400x200 elements of 100 m, NGLL=5, 6000 steps"
    elif args.workload == "psv_rsf":
        pair = workloads.psv_rsf(scale=args.scale, precision=prec, **kw)
        name = "P-SV rate-and-state rupture (aging), von Karman medium, 1024x512 elements, NGLL=5"
    elif args.workload == "tpv3_inplane":
        # the reference's TPV3 in-plane example refined 8x in each direction
        pair = workloads.tpv3_inplane(scale=8.0 * args.scale, precision=prec, **kw)
        name = ("SCEC TPV3 in-plane example refined 8x: 560x320 elements, NGLL=6, Newmark, Kelvin-Voigt band, "
                "one-sided SWF fault, Dirichlet side, 16 s")
    else:
        pair = workloads.plain_psv(scale=args.scale, precision=prec)
        name = "plain P-SV elastic, 100x100 elements of 100 m, NGLL=5, 2000 steps"
    if args.scale != 1.0:
        name += " (scale %.3g)" % args.scale
    return pair, name


def make_workload(args):
    from sem2dpack_gb300 import workloads
    pair, name = workload_deck(args)
    return workloads.build(pair), name


def desc_bytes(d):
    """Bytes of every host array the descriptor hands to sem2d_gpu_create."""
    n2, ne, npn, nd, nf = d.ngll * d.ngll, d.nelem, d.npoin, d.ndof, d.nflt
    sizes = {"ibool": 4 * n2 * ne, "coord": 16 * npn, "hprime": 8 * n2, "wgll": 8 * d.ngll,
             "rmass": 8 * npn * nd, "abs_node": 4 * d.nabs, "abs_C": 8 * d.nabs * nd,
             "src_node": 4 * d.nsrc, "src_dir": 16 * d.nsrc, "rec_node": 4 * d.nrec}
    for f in ("Kx", "Kz", "la", "mu", "mux"):
        sizes[f] = 8 * n2 * ne
    if nf:
        sizes["fault"] = 8 * nf * (2 + 2 + 1 + 3 * nd + 2 + 1 + 5) + 8 * nf
    return sum(sizes.values())


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="sem2d_clocks_rank%d_" % self.index, suffix=".csv")
            self.f = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        try:
            os.unlink(self.path)
        except OSError:
            pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    for path in (os.path.join(ROOT, "MEASURED_PEAKS.json"),):
        if os.path.exists(path):
            with open(path) as f:
                return json.load(f), "measured"
    return {"hbm_gbs": 6800.0}, "fallback"


MARCH_TX = 31  # element columns of a unit of the march kernels


def ncu_traffic(kernel, workload, npoin):
    """DRAM bytes per launch of `kernel` from the committed ncu summary of a
    (possibly smaller) capture of the workload, scaled by the node count."""
    path = os.path.join(ROOT, "profiles", "%s_%s.txt" % (kernel, workload))
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_node:"):
            try:
                return float(line.split(":", 1)[1].split()[0]) * npoin
            except ValueError:
                return None
    return None


def cpu_baseline(desc, owner, npoin, seconds):
    """FP64 oracle (single thread) on a bounded sample of the workload."""
    from oracle import pyoracle as po
    sim = po.OracleSim(desc, owner=owner)
    t0 = time.perf_counter()
    sim.run(2)
    rate = 2 / max(time.perf_counter() - t0, 1e-9)
    n = max(2, min(int(rate * seconds), desc.nt - 2))
    t0 = time.perf_counter()
    sim.run(n)
    dt = time.perf_counter() - t0
    return npoin * n / dt, n


def run_reference(args, rank):
    """The reference's CPU path (its FP64 restatement: the reference is
    Fortran and no Fortran compiler exists here) on the workload of the
    GB300 arm, set up by the oracle's own restated init (no product library
    is loaded).  Each benchmark step is a bounded sample of the workload's
    time steps; independent problems run one per host thread."""
    if rank != 0:
        return
    from concurrent.futures import ThreadPoolExecutor

    from oracle import pyoracle as po
    from sem2dpack_gb300 import workloads
    threads = 1
    if args.workload == "batch_shots":
        decks = workloads.batch_shots(nsim=args.nsim, scale=args.scale, nsteps=3000)
        sizes = [(dk.nelem[0] * 4 + 1) * (dk.nelem[1] * 4 + 1) for dk in decks]
        name = batch_name(len(decks), sum(sizes), args.scale)
        threads = max(1, min(os.cpu_count() or 1, 16))
        # a seeded sample of the shots, one per host thread
        import numpy as np
        pick = np.random.default_rng(20261203).choice(len(decks), size=min(threads, len(decks)), replace=False)
        setups = [po.OracleSetup(decks[int(i)]) for i in pick]
        what = "%d of the %d shots (seeded sample), one per host thread" % (len(setups), len(decks))
        nprob = len(decks)
    else:
        pair, name = workload_deck(args, grid_cls=OracleGrid)
        setups = [po.OracleSetup(pair[0] if isinstance(pair, tuple) else pair)]
        what = name
        nprob = 1
    sims = []
    for S in setups:
        d = S.desc()
        d.precision = 0
        sims.append((po.OracleSim(d, owner=S), d.npoin, d.nt))
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda s: s[0].run(2), sims))
    rate = 2 / max(time.perf_counter() - t0, 1e-9)
    nt_min = min(s[2] for s in sims)
    per = max(1, min(int(rate * 2.0), (nt_min - 2) // max(1, args.steps + args.warmup)))

    def bench_step():
        with ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(lambda s: s[0].run(per), sims))

    for _ in range(args.warmup):
        bench_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bench_step()
    el = time.perf_counter() - t0
    value = sum(n for _, n, _ in sims) * per * args.steps / el
    sample = "%d time steps per benchmark step of %s, FP64, %d thread(s)" % (per, what, threads)
    print(json.dumps({
        "impl": "reference", "metric": "GLL node-steps/s", "value": value, "unit": "node-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": name, "global_batch": len(sims), "seq_len": 0, "parallelism": "replicas",
                   "reference_build": "CPU restatement of the reference's step (oracle), set up by its own "
                                      "restated init; the Fortran reference needs a Fortran compiler"},
        "cpu_baseline": {"value": value, "unit": "node-steps/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "node-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def batch_parts(nt, k):
    """Time steps of each of the k benchmark steps that together make one
    complete nt-step solve."""
    k = max(1, min(k, nt))
    return [nt // k + (1 if i < nt % k else 0) for i in range(k)]


# problems built and uploaded per group of the batched workload: the host
# holds one group (about 11 GB of arrays for 64 shots) at a time
BUILD_GROUP = 64


def built_groups(decks, workers, group, build_s):
    """Problems of the decks in order, built `group` at a time on `workers`
    host threads; a group is built only when the previous one has been
    taken (BatchSolver uploads each group with one batch_add_many call, so
    building and uploading do not compete for the host threads).  The
    building time is added to build_s[0]."""
    from concurrent.futures import ThreadPoolExecutor

    from sem2dpack_gb300 import workloads
    with ThreadPoolExecutor(max_workers=workers) as ex:
        for k in range(0, len(decks), group):
            t0 = time.perf_counter()
            probs = list(ex.map(workloads.build, decks[k:k + group]))
            build_s[0] += time.perf_counter() - t0
            while probs:
                yield probs.pop(0)


def oracle_sample(decks, nsteps_of, threads):
    """Runs the FP64 oracle (CPU restatement of the reference's step, one
    problem per host thread, as independent reference runs would) on the
    given decks; returns (node-steps, wall seconds, [seismograms])."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import pyoracle as po
    sims = []
    for dk in decks:
        S = po.OracleSetup(dk)
        d = S.desc()
        d.precision = 0
        sims.append((po.OracleSim(d, owner=S), d.npoin, nsteps_of(d)))
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda s: s[0].run(s[2]), sims))
    wall = time.perf_counter() - t0
    return sum(n * k for _, n, k in sims), wall, [s[0].seismograms() for s in sims]


def batch_name(nsim, npoin, scale):
    name = ("batched P-SV shots: %d problems of 64^2..512^2 elements (25 m), NGLL=5, 3-8 layer media, "
            "Ricker force, 32 receivers, 3000 steps, %d GLL nodes in total" % (nsim, npoin))
    if scale != 1.0:
        name += " (scale %.3g)" % scale
    return name


def run_batch(args, rank, world, local, torch, dist, barrier):
    """The batched-shot configuration: 256 uneven P-SV problems stepped by
    one launch per time step (sem2d_gpu_batch_* path), all 3000 time steps
    of the solve timed: the K benchmark steps are consecutive parts of one
    complete solve from rest."""
    import numpy as np

    from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, BatchSolver, workloads
    prec = PRECISION_MIXED if args.precision == "mixed" else PRECISION_FP64
    decks = workloads.batch_shots(nsim=args.nsim, scale=args.scale, nsteps=3000, precision=prec)
    nt = min(args.time_steps or 3000, 3000)
    workers = max(1, min(16, os.cpu_count() or 1))
    t0 = time.perf_counter()
    build_s = [0.0]
    sim = BatchSolver(built_groups(decks, workers, BUILD_GROUP, build_s), group=BUILD_GROUP)
    setup_s = time.perf_counter() - t0
    build_s = build_s[0]
    descs = [m.desc for m in sim.members]
    npoin = sum(d.npoin for d in descs)
    h2d = sum(desc_bytes(d) for d in descs)
    d2h = sum(8 * d.rec_nsamp * d.nrec * d.ndof for d in descs)
    dtype = "f32" if prec == PRECISION_MIXED else "f64"
    name = batch_name(len(sim), npoin, args.scale)
    stream = torch.cuda.ExternalStream(sim.stream)

    # end to end through the C-ABI from host arrays: the upload
    # (sem2d_gpu_batch_add_many per group), one complete solve,
    # every member's seismograms back, and (below) the destroy
    barrier()
    t0 = time.perf_counter()
    sim.step(nt)
    sis_gpu = [m.seismograms() for m in sim.members]
    t_run = time.perf_counter() - t0

    # device-resident: warm-up parts, then one complete solve from rest in
    # K parts, events around each part and around every kernel launch
    parts = batch_parts(nt, args.steps)
    sim.reset()
    left = nt
    for _ in range(args.warmup):
        if left < parts[0]:
            sim.reset()
            left = nt
        sim.step(parts[0])
        left -= parts[0]
    sim.sync()
    sim.reset()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = sim.launches
    ms, bulk = [], 0.0
    for n in parts:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        kms = sim.step_timed(n)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        bulk += kms[0]
    launches = sim.launches - l0
    barrier()
    clk = clocks.stop()
    total = sum(ms)
    if dist is not None:
        t = torch.tensor([total], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total = float(t.item())
    value = world * npoin * nt / (total / 1000.0)
    bulk_ms = bulk / nt
    bpn = BYTES_PER_NODE_STEP[(2, dtype)]
    achieved = npoin * bpn / (bulk_ms / 1000.0) / 1e9
    peaks, peak_kind = measured_peaks()
    shape = sim.tile
    kernel = "march_batch_kernel" if shape[0] == MARCH_TX else "strip_batch_kernel"
    traffic = ncu_traffic(kernel, "batch_shots", npoin)
    t0 = time.perf_counter()
    sim.close()
    t_close = time.perf_counter() - t0
    e2e_value = world * npoin * nt / (sim.upload_seconds + t_run + t_close)

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the smallest shots, all their time steps, one per host thread
        order = np.argsort([d.npoin for d in descs])
        threads = max(1, min(os.cpu_count() or 1, 16))
        pick = [int(i) for i in order[:threads]]
        ns, wall, sis_ref = oracle_sample([decks[i] for i in pick], lambda d: nt, threads)
        err = max(float(np.linalg.norm(sis_gpu[i] - r) / np.linalg.norm(r)) for i, r in zip(pick, sis_ref))
        base = {"value": ns / wall, "unit": "node-steps/s", "cores": threads, "kind": "port",
                "sample": "the %d smallest of the %d shots (%d GLL nodes), all %d time steps each, FP64, "
                          "one shot per host thread" % (len(pick), len(descs), sum(descs[i].npoin for i in pick), nt),
                "sample_seconds": wall,
                "seismogram_rel_l2_max": err,
                "seismogram_rel_l2_note": "GPU mixed-precision seismograms of the sampled shots against this FP64 "
                                          "oracle run, all time steps"}

    fp64 = None
    if rank == 0 and not args.no_fp64_plain:
        fp64 = fp64_plain_record(torch, barrier)

    if rank == 0:
        print(json.dumps({
            "metric": "GLL node-steps/s", "value": value, "unit": "node-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / len(parts),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic",
            "config": {"workload": name, "global_batch": len(descs), "seq_len": 0,
                       "parallelism": "replicas", "npoin": npoin,
                       "time_steps_timed": nt, "time_steps_per_step": nt / len(parts),
                       "timed_region": "one complete %d-step solve of every shot from rest, in %d consecutive "
                                       "benchmark steps" % (nt, len(parts)),
                       "precision": "FP32 fields" if dtype == "f32" else "FP64",
                       "l2": "inputs larger than L2 (the batch's fields are %.1f GB)" % (npoin * bpn / 1e9),
                       "host_setup_s": setup_s, "host_build_s": build_s,
                       "launch_shape": {"element_columns": shape[0], "chunk_rows": shape[1]}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks.get("hbm_gbs"),
                         "unit": "GB/s", "frac": achieved / peaks.get("hbm_gbs"),
                         "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": kernel, "bytes_per_node_step": bpn,
                         "bulk_ms_per_launch": bulk_ms,
                         "launch_timing": "CUDA events around every launch of the timed solve"},
            "cpu_baseline": base,
            "e2e": {"value": e2e_value, "unit": "node-steps/s",
                    "h2d_bytes_per_step": h2d / len(parts), "d2h_bytes_per_step": d2h / len(parts),
                    "h2d_bytes_per_solve": h2d, "d2h_bytes_per_solve": d2h,
                    "upload_s": sim.upload_seconds, "run_s": t_run, "destroy_s": t_close,
                    "path": "BatchSolver through the C-ABI: sem2d_gpu_batch_add_many of every shot from host "
                            "arrays in groups of %d (members set up on host threads), one complete solve, all "
                            "seismograms back, destroy" % BUILD_GROUP},
            "fp64_plain": fp64,
            "clocks": clk,
            "gpu_launches": launches,
        }), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def fp64_plain_record(torch, barrier):
    """The plain FP64 P-SV box (100 x 100 elements, NGLL=5, 2000 steps):
    the FP64 GPU path beside the mixed-precision headline."""
    from sem2dpack_gb300 import PRECISION_FP64, Solver, workloads
    P = workloads.build(workloads.plain_psv(precision=PRECISION_FP64))
    d = P.desc()
    sim = Solver(d, owner=P)
    stream = torch.cuda.ExternalStream(sim.stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ms = []
    for k in range(4):
        sim.reset()
        flush.fill_(1.0)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.step(d.nt)
        e1.record(stream)
        e1.synchronize()
        if k:
            ms.append(e0.elapsed_time(e1))
    sim.sync()
    sim.close()
    best = min(ms)
    return {"workload": "plain P-SV elastic, 100x100 elements of 100 m, NGLL=5, 2000 steps, FP64",
            "value": d.npoin * d.nt / (best / 1000.0), "unit": "node-steps/s", "ms_per_solve": best,
            "npoin": d.npoin, "solves_timed": len(ms)}


def run_gradient(args, rank, world, local, torch, dist, barrier):
    """Gradient workflow (8 shots on 512^2 elements): forward solves against
    forward-with-checkpoints + adjoint; reports the cost ratio."""
    import ctypes as C

    import numpy as np

    from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Solver, workloads
    from sem2dpack_gb300._lib import lib
    prec = PRECISION_MIXED if args.precision == "mixed" else PRECISION_FP64
    nt = args.time_steps or 4000
    models, start, true = workloads.gradient_shots(scale=args.scale, nsteps=nt, precision=prec)
    every = max(1, int(round(np.sqrt(nt))))
    pp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    sims, obs = [], []
    t_create, h2d = 0.0, 0
    for m in models:
        Pt = workloads.build(m.deck_for(*true))
        st = Solver(Pt)
        st.step(nt)
        obs.append(st.seismograms())
        st.close()
        P = workloads.build(m.deck_for(*start))
        d = P.desc()
        d.precision = prec
        d.adjoint = 1
        t0 = time.perf_counter()
        sims.append((Solver(d, owner=P), d))
        t_create += time.perf_counter() - t0
        h2d += desc_bytes(d)
    npoin = sims[0][1].npoin
    grads = [np.zeros(npoin) for _ in range(3)]

    def forward_only():
        for s, _ in sims:
            s.reset()
            s._check(lib().sem2d_gpu_checkpoint_every(s.h, 0))
        barrier()
        t0 = time.perf_counter()
        for s, _ in sims:
            s.step(nt)
        for s, _ in sims:
            s.sync()
        return time.perf_counter() - t0

    def gradient():
        for s, _ in sims:
            s.reset()
            s._check(lib().sem2d_gpu_checkpoint_every(s.h, every))
        barrier()
        t0 = time.perf_counter()
        for k, (s, d) in enumerate(sims):
            s.step(nt)
            r = np.asfortranarray(s.seismograms() - obs[k])
            s._check(lib().sem2d_gpu_adjoint(s.h, pp(r), pp(grads[0]), pp(grads[1]), pp(grads[2])))
        return time.perf_counter() - t0

    # end to end: the uploads (timed at creation), one forward solve of every
    # shot, the seismograms back
    barrier()
    t0 = time.perf_counter()
    for s, _ in sims:
        s.reset()
        s.step(nt)
    for s, _ in sims:
        s.seismograms()
    e2e_value = world * len(sims) * sims[0][1].npoin * nt / (t_create + time.perf_counter() - t0)
    d2h = sum(8 * d.rec_nsamp * d.nrec * d.ndof for _, d in sims)
    for _ in range(max(1, args.warmup)):
        forward_only()
        gradient()
    clocks = ClockSampler(local)
    clocks.start()
    tf = [forward_only() for _ in range(args.steps)]
    tg = [gradient() for _ in range(args.steps)]
    clk = clocks.stop()
    l0 = sum(s.launches for s, _ in sims)
    fwd = min(tf)
    grd = min(tg)
    value = len(sims) * npoin * nt / fwd
    name = ("gradient workflow: %d P-SV shots on %dx%d elements of 25 m, NGLL=5, %d of 4000 steps, "
            "checkpoint every %d steps" % (len(sims), models[0].deck.nelem[0], models[0].deck.nelem[1], nt, every))
    # the bound from the bytes a step moves per node (P-SV FP32): forward 44,
    # recomputed forward with its ring of d, v, a 68, reverse step 92 (the
    # (lambda, w) step 60: lambda, w read and written, moduli, inverse mass,
    # a^n, the mass sum; the moduli pass 32: lambda^n, d^n, the two sums)
    bound = (44 + 68 + 60 + 32) / 44
    # aggregate roofline of the forward solves: 44 B per node-step over
    # their wall time, and of the whole gradient: the 204 B its three
    # phases move per node-step over its wall time
    peaks, peak_kind = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    fwd_gbs = len(sims) * npoin * nt * 44 / fwd / 1e9
    grd_gbs = len(sims) * npoin * nt * (44 + 68 + 60 + 32) / grd / 1e9
    if rank == 0:
        print(json.dumps({
            "metric": "GLL node-steps/s", "value": value, "unit": "node-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * fwd,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if prec == PRECISION_MIXED else "f64", "data": "synthetic",
            "config": {"workload": name, "global_batch": len(sims), "seq_len": 0, "parallelism": "replicas",
                       "npoin": npoin, "time_steps_per_step": nt},
            "gradient_cost": {"forward_s": fwd, "forward_and_adjoint_s": grd, "ratio": grd / fwd,
                              "bytes_bound": bound,
                              "note": "forward with checkpoints + segment recomputation + adjoint, "
                                      "over the plain forward solves of the same shots; bytes_bound: the "
                                      "ratio of the bytes per node the three phases move to a forward step's"},
            "roofline": {"bound": "hbm", "achieved": fwd_gbs, "peak": hbm, "unit": "GB/s",
                         "frac": fwd_gbs / hbm if hbm else None, "traffic": None, "peak_kind": peak_kind,
                         "note": "forward solves of the 8 shots, 44 B per node-step over their wall time",
                         "gradient_achieved": grd_gbs,
                         "gradient_frac": grd_gbs / hbm if hbm else None},
            "cpu_baseline": None,
            "e2e": {"value": e2e_value, "unit": "node-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "path": "Solver creation of every shot from host arrays, one "
                                                       "forward solve each, seismograms back"},
            "clocks": clk, "gpu_launches": l0,
        }), flush=True)
    for s, _ in sims:
        s.close()


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    if args.workload == "batch_shots":
        run_batch(args, rank, world, local, torch, dist, barrier)
        return
    if args.workload == "gradient_shots":
        run_gradient(args, rank, world, local, torch, dist, barrier)
        return
    from sem2dpack_gb300 import Solver
    prob, name = make_workload(args)
    desc = prob.desc()
    npoin, nt, ndof = desc.npoin, desc.nt, desc.ndof
    cut = None
    if args.time_steps:
        nt = min(nt, args.time_steps)
    elif args.workload == "psv_rsf":
        # the synthetic rate-and-state rupture cannot reach its 10000th step:
        # it runs supershear as a crack whose slip rate grows to 25 m/s, and
        # at step 5000 (t = 5.9 s) a node needs more than the reference's 200
        # Newton iterations (where the reference aborts); halving dt moves
        # that only to t = 6.3 s.  The first 4000 steps are timed.
        nt = min(nt, 4000)
        cut = ("first 4000 of 10000 steps: the aging-law rupture grows to slip rates of 25 m/s and a "
               "node exceeds the 200 Newton iterations of the reference at step 5000 (t = 5.9 s)")
    dtype = "f32" if desc.precision == 1 else "f64"
    sim = Solver(desc, owner=prob)
    stream = torch.cuda.ExternalStream(sim.stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)

    def one_solve(timed):
        sim.reset()
        flush.fill_(1.0)
        barrier()
        if not timed:
            sim.step(nt)
            sim.sync()
            return 0.0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.step(nt)
        e1.record(stream)
        e1.synchronize()
        sim.sync()
        return e0.elapsed_time(e1)

    for _ in range(args.warmup):
        one_solve(False)
    clocks = ClockSampler(local)
    clocks.start()
    l0 = sim.launches
    ms = [one_solve(True) for _ in range(args.steps)]
    launches = sim.launches - l0
    clk = clocks.stop()
    total = sum(ms)
    if dist is not None:
        t = torch.tensor([total], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total = float(t.item())
    value = world * npoin * nt * args.steps / (total / 1000.0)

    # per-kernel durations (events around every launch) for the roofline
    sim.reset()
    kms = sim.step_timed(nt)
    bulk_ms = kms[0] / nt
    bpn = BYTES_PER_NODE_STEP[(ndof, dtype)]
    if args.workload == "tpv3_inplane":
        # Newmark: + read/write of the accelerations; Kelvin-Voigt: + eta
        bpn = (4 if dtype == "f32" else 8) * (4 + 4 + 4 + 1 + 2 + 1)
    achieved = npoin * bpn / (bulk_ms / 1000.0) / 1e9
    peaks, peak_kind = measured_peaks()
    kernel = "march_step_kernel" if sim.tile[0] == MARCH_TX else "strip_step_kernel"
    traffic = ncu_traffic(kernel, args.workload, npoin)

    # end to end through the C-ABI from host buffers
    sim.close()
    del stream
    h2d = desc_bytes(desc)
    nflt_onx = (desc.flt_oixn - desc.flt_oix1) // max(desc.flt_oixd, 1) + 1 if desc.nflt else 0
    d2h = 8 * desc.rec_nsamp * desc.nrec * ndof + 8 * nflt_onx * 6 * desc.flt_nsamp
    e2e_times = []
    for _ in range(2):
        barrier()
        t0 = time.perf_counter()
        s2 = Solver(desc, owner=prob)
        s2.step(nt)
        s2.seismograms()
        if desc.nflt:
            s2.fault_series()
        s2.close()
        e2e_times.append(time.perf_counter() - t0)
    e2e_value = world * npoin * nt / min(e2e_times)

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, n = cpu_baseline(desc, prob, npoin, args.cpu_seconds)
        base = {"value": v, "unit": "node-steps/s", "cores": 1, "kind": "port",
                "sample": "%d of %d time steps of the same workload in FP64 on 1 host thread" % (n, nt)}

    if rank == 0:
        line = {
            "metric": "GLL node-steps/s", "value": value, "unit": "node-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic",
            "config": {"workload": name, "global_batch": 1, "seq_len": 0, "parallelism": "replicas",
                       "npoin": npoin, "time_steps_per_step": nt,
                       "precision": "FP32 fields, FP64 fault state" if dtype == "f32" else "FP64",
                       "l2": "512 MB buffer written before every timed solve; " + (
                           "the solve's working set (%.0f MB) then stays L2-resident across its time steps"
                           if npoin * bpn < 100e6 else "the fields (%.0f MB) are larger than L2") % (npoin * bpn / 1e6),
                       **({"time_steps_cut": cut} if cut else {})},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks.get("hbm_gbs"),
                         "unit": "GB/s", "frac": achieved / peaks.get("hbm_gbs"),
                         "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": kernel, "bytes_per_node_step": bpn,
                         "bulk_ms_per_launch": bulk_ms, "fault_ms_per_launch": kms[1] / nt,
                         "receiver_ms_per_launch": kms[2] / nt},
            "cpu_baseline": base,
            "e2e": {"value": e2e_value, "unit": "node-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "clocks": clk,
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""Benchmark: batched 3D surface-wave rjMCMC forward evaluations on one GB300.

Workload (the batched surface-wave configuration): 64 chains, grid
41 x 41 x 31 over 40 x 40 x 6 km, per-chain Voronoi cell counts uniform on
[10, 400], Vs uniform on [0.3, 2.5] km/s, Vp = 1.73 Vs, density 2.0 g/cc,
20 Rayleigh fundamental-mode phase-velocity periods log-spaced 0.5-5 s,
50 stations, 1,225 paths per period, sigma = 2% of the travel time. Every
step evaluates one move proposal per chain (one Voronoi nucleus displaced),
then commits it, so each proposal's dispersion work is the columns its cell
change touches, as in the reference.

value  = proposal evaluations / s with the proposals already resident in HBM
         (device API, CUDA-event timed).
e2e    = the same through the host API (mct_surf_forward / mct_surf_commit):
         pinned host buffers copied in and results copied out every step.
plain  = one chain per call through the host API (the per-proposal drop-in).

--impl reference times the CPU restatement of the reference's path (oracle/)
on the host cores on a bounded sample of the same workload.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# DRAM bytes (read + write) of the fm2d stage of one forward of the surface
# workload below (refine_slowness 0.223 GB, refined solves 1.510 GB, coarse
# solves 0.220 GB), measured with ncu's one-pass dram__bytes_read.sum and
# dram__bytes_write.sum over the stage's launches of the bench's first forward
FM2D_DRAM_BYTES_PER_FORWARD = 1.953e9
NCHAINS = 64
NCELL_MAX = 400
SEED = 20261203
METRIC = "forward evals/s & p99 latency: served batch vs plain, 1 GB300, ttime err<=1e-4"
CONFIG = {"workload": "batched 3D surface-wave rjMCMC: 64 chains, 41x41x31 grid over 40x40x6 km, "
                      "10-400 Voronoi cells/chain, 20 Rayleigh phase periods 0.5-5 s, 50 stations, "
                      "1225 paths/period, move proposals committed each step",
          "chains": NCHAINS, "grid": [41, 41, 31], "periods": 20, "stations": 50,
          "paths_per_period": 1225, "dispersion_root_search": "FP32 bracketing + FP64 polish",
          "fm2d": "reference marching order, FP64 updates in the reference's operation order",
          "l2": "flushed (512 MB write) between steps"}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); smax.append(float(f[2])); power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def job_rate(units_per_rank, elapsed_ms, ws, device=None):
    """Whole-job throughput over ws replica ranks: the units all ranks
    processed over the slowest rank's time (all-reduce MAX of the elapsed
    time). Returns (rate per second, max elapsed ms)."""
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(elapsed_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    return units_per_rank * ws / (elapsed_ms / 1e3), elapsed_ms


def make_workload(steps_total):
    from mctomo_gb300 import synthetic
    rng = np.random.default_rng(SEED)
    grid, settings, data = synthetic.surface_workload(rng)
    ncells, pts, par = synthetic.surface_chain_models(rng, NCHAINS, NCELL_MAX, grid)
    props = []
    cur_p, cur_q = pts, par
    for _ in range(steps_total):
        cur_p, cur_q = synthetic.perturb_chain_models(rng, ncells, cur_p, cur_q, grid)
        props.append((cur_p, cur_q))
    npd = len(data["freqs"])
    n0 = np.full((NCHAINS, npd), 0.02)
    n1 = np.zeros((NCHAINS, npd))
    return grid, settings, data, ncells, (pts, par), props, n0, n1


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)["hbm_gbs"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def run_gpu(args):
    import torch
    from mctomo_gb300 import SurfaceLikelihood, lib
    from mctomo_gb300._lib import check
    ws, rank = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    dev = torch.device("cuda")
    K, W = args.steps, args.warmup
    grid, settings, data, ncells, init, props, n0, n1 = make_workload(K + W + 1)
    settings = dict(settings, precision=1, tt_precision=args.tt_precision)
    lk = SurfaceLikelihood(grid, settings, data, nslots=NCHAINS, ncell_max=NCELL_MAX)
    L = lib()
    slots = np.arange(NCHAINS, dtype=np.int32)
    # initial state (every column computed), committed
    lk.forward(slots, ncells, init[0], init[1], n0, n1)
    lk.commit(np.ones(NCHAINS, np.int32))
    # device-resident proposals
    stream_p = ctypes.c_void_p()
    check("mct_surf_stream", L.mct_surf_stream(lk.h, ctypes.byref(stream_p)))
    ext = torch.cuda.ExternalStream(stream_p.value)
    d_slots = torch.from_numpy(slots).to(dev)
    d_ncells = torch.from_numpy(ncells).to(dev)
    d_n0 = torch.from_numpy(n0).to(dev)
    d_n1 = torch.from_numpy(n1).to(dev)
    d_acc = torch.ones(NCHAINS, dtype=torch.int32, device=dev)
    d_out = torch.zeros((NCHAINS, 4), dtype=torch.float64, device=dev)
    d_pts = [torch.from_numpy(p).to(dev) for p, _ in props]
    d_par = [torch.from_numpy(q).to(dev) for _, q in props]
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()

    def dstep(i):
        rc = L.mct_surf_forward_device(lk.h, NCHAINS, d_slots.data_ptr(), d_ncells.data_ptr(),
                                       d_pts[i].data_ptr(), d_par[i].data_ptr(), d_n0.data_ptr(),
                                       d_n1.data_ptr(), d_out.data_ptr(), None)
        check("mct_surf_forward_device", rc)
        check("mct_surf_commit_device", L.mct_surf_commit_device(lk.h, d_acc.data_ptr(), None))

    for i in range(W):
        dstep(i)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    check("mct_surf_profile_start", L.mct_surf_profile_start(lk.h, K))
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    step_ms = []
    with torch.cuda.stream(ext):
        for i in range(W, W + K):
            flush.fill_(i & 0xff)
            e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            dstep(i)
            e1.record(ext)
            step_ms.append((e0, e1))
    torch.cuda.synchronize()
    cl = clocks.stop()
    times = [a.elapsed_time(b) for a, b in step_ms]
    total_ms = sum(times)
    stage = (ctypes.c_double * 4)()
    nsteps = ctypes.c_int()
    launches = ctypes.c_longlong()
    check("mct_surf_profile_read", L.mct_surf_profile_read(lk.h, stage, ctypes.byref(nsteps), ctypes.byref(launches)))
    check("mct_surf_profile_start", L.mct_surf_profile_start(lk.h, 0))
    out = d_out.cpu().numpy()
    value, total_ms = job_rate(NCHAINS * K, total_ms, ws, dev)

    # end to end through the host API, pinned host buffers
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    hp = [(pin(p), pin(q)) for p, q in props]
    e2e_ms = []
    lk.forward(slots, ncells, hp[0][0], hp[0][1], n0, n1)
    lk.commit(np.ones(NCHAINS, np.int32))
    for i in range(W, W + K):
        flush.fill_(i & 0xff)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        o = lk.forward(slots, ncells, hp[i][0], hp[i][1], n0, n1)
        lk.commit(np.ones(NCHAINS, np.int32))
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_value, _ = job_rate(NCHAINS * len(e2e_ms), sum(e2e_ms), ws, dev)
    h2d = NCHAINS * NCELL_MAX * 3 * 8 * 2 + NCHAINS * (4 + 4) + 2 * NCHAINS * n0.shape[1] * 8 + NCHAINS * 4
    d2h = NCHAINS * 4 * 8

    # plain drop-in: one chain per call
    plain_ms = []
    nplain = min(64, NCHAINS)
    for c in range(nplain):
        t0 = time.perf_counter()
        lk.forward(slots[c:c + 1], ncells[c:c + 1], hp[W + K][0][c:c + 1], hp[W + K][1][c:c + 1],
                   n0[c:c + 1], n1[c:c + 1])
        lk.commit(np.ones(1, np.int32))
        plain_ms.append((time.perf_counter() - t0) * 1e3)
    plain_value, _ = job_rate(len(plain_ms), sum(plain_ms), ws, dev)

    # roofline of the dominant stage (fm2d travel times): algorithmic bytes =
    # for every (chain, period, source) solve, each node of the 41x41 grid read
    # (velocity) and written (travel time) once in FP64 = 16 B/node/solve
    stage_ms = [stage[k] / max(nsteps.value, 1) for k in range(4)]
    names = ["gridding", "layering+dispersion", "fm2d travel times", "misfit"]
    dom = int(np.argmax(stage_ms))
    nsolve = NCHAINS * sum(1 for p in range(20) for s in range(50)
                           if (np.asarray(data["raystat"][p]).reshape(50, 50)[s].any() or s == 0))
    alg_bytes = {2: nsolve * 41 * 41 * 16.0,
                 0: NCHAINS * (41 * 41 * 31 * (4 + 24)) + NCHAINS * 400 * 48.0,
                 1: 0.0, 3: NCHAINS * 20 * 1225 * 24.0}[dom]
    peak, peak_kind = peaks()
    achieved = alg_bytes / (stage_ms[dom] / 1e3) / 1e9 if alg_bytes else 0.0
    # measured DRAM traffic of the FP64 fm2d stage (FM2D_DRAM_BYTES_PER_FORWARD)
    traffic = FM2D_DRAM_BYTES_PER_FORWARD if dom == 2 and args.tt_precision == 0 else None
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "proposal evals/s", "n_gpus": ws,
        "steps": K, "warmup": W, "ms_per_step": round(total_ms / K, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 dispersion polish; f32 dispersion bracketing; " + (
            "f64 fm2d in the reference's operation order (times identical to the reference)" if args.tt_precision == 0
            else "double-float (f32 pairs) fm2d"),
        "data": "synthetic (seeded, shapes of the configuration)",
        "config": CONFIG if args.tt_precision == 0 else dict(CONFIG, fm2d="reference marching order, " + (
            "double-float (FP32 pair) updates" if args.tt_precision == 1 else "int32 fixed-point times")),
        "e2e": {"value": round(e2e_value, 3), "unit": "proposal evals/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "plain": {"value": round(plain_value, 3), "unit": "proposal evals/s", "p50_ms": round(float(np.percentile(plain_ms, 50)), 3),
                  "p99_ms": round(float(np.percentile(plain_ms, 99)), 3)},
        "batched_latency_ms": {"p50": round(float(np.percentile(times, 50)), 3),
                               "p99": round(float(np.percentile(times, 99)), 3)},
        "stage_ms_per_step": {n: round(v, 4) for n, v in zip(names, stage_ms)},
        "roofline": {"kernel": names[dom], "bound": "hbm", "achieved": round(achieved, 3), "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 6),
                     "traffic": traffic,
                     # what actually limits the stage (HBM is ~0 % busy): the
                     # latency of the reference's sequential heap march, one
                     # node after another per solve; ncu --set full on the
                     # small fm2d case (--case fm2d --case-precision 0
                     # --case-maps 64: 3,136 solves)
                     "limiter": "latency of the sequential heap march (heap warp + FP64 update warp per solve)",
                     "ncu_small_case": {"issue_active": {"coarse": 0.270, "refined": 0.257},
                                        "fp64_pipe_active": {"coarse": 0.430, "refined": 0.385},
                                        "resident_solves_per_sm": 16, "dram_throughput": 0.001}},
        "gpu_launches": int(launches.value),
        "clocks": cl,
        "valid_models": int((out[:, 3] == 0).sum()),
    }
    collected = []
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(grid, settings, data, ncells, init, props, n0, n1, args, collected)
        try:
            line["accuracy"] = surface_accuracy(grid, settings, data, ncells, init, props, n0, n1, collected)
        except Exception as e:   # the throughput line stands without it
            line["accuracy"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if rank == 0 and args.tt_precision == 0 and not args.no_variant:
        # the double-float fm2d variant on the same proposals, device path
        vs = dict(settings, tt_precision=1)
        lk2 = SurfaceLikelihood(grid, vs, data, nslots=NCHAINS, ncell_max=NCELL_MAX)
        lk2.forward(slots, ncells, init[0], init[1], n0, n1)
        lk2.commit(np.ones(NCHAINS, np.int32))
        sp2 = ctypes.c_void_p()
        check("mct_surf_stream", L.mct_surf_stream(lk2.h, ctypes.byref(sp2)))
        ext2 = torch.cuda.ExternalStream(sp2.value)

        def vstep(i):
            check("mct_surf_forward_device", L.mct_surf_forward_device(
                lk2.h, NCHAINS, d_slots.data_ptr(), d_ncells.data_ptr(), d_pts[i].data_ptr(), d_par[i].data_ptr(),
                d_n0.data_ptr(), d_n1.data_ptr(), d_out.data_ptr(), None))
            check("mct_surf_commit_device", L.mct_surf_commit_device(lk2.h, d_acc.data_ptr(), None))
        for i in range(W):
            vstep(i)
        torch.cuda.synchronize()
        ev = []
        with torch.cuda.stream(ext2):
            for i in range(W, W + K):
                flush.fill_(i & 0xff)
                e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
                e0.record(ext2)
                vstep(i)
                e1.record(ext2)
                ev.append((e0, e1))
        torch.cuda.synchronize()
        vms = sum(a.elapsed_time(b) for a, b in ev)
        lk2.close()
        var = {"value": round(NCHAINS * K / (vms / 1e3), 3), "unit": "proposal evals/s",
               "ms_per_step": round(vms / K, 4), "fm2d": "double-float (f32 pairs) updates"}
        if collected:
            try:
                var["accuracy"] = surface_accuracy(grid, vs, data, ncells, init, props, n0, n1, collected)
            except Exception as e:
                var["accuracy"] = {"error": "%s: %s" % (type(e).__name__, e)}
        line["variants"] = {"double_float_fm2d": var}
    if rank == 0:
        print(json.dumps(line), flush=True)
    lk.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def cpu_sample(grid, settings, data, ncells, init, props, n0, n1, nprop, threads, collect=None):
    """Times the oracle's restatement of the reference path on nprop proposals
    (one chain each), each against its chain's committed state: only the
    columns whose model changed get new dispersion curves, as the reference's
    CGAL box arranges. The timed call includes the chain's kd-tree gridding.
    With collect (a list), each proposal's (chain, travel times, phase maps,
    out) are appended for the accuracy check."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle
    orc = oracle.load()
    P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    f = lambda a, t=np.float64: np.ascontiguousarray(a, t)  # noqa: E731
    gi = np.array([grid["nx"], grid["ny"], grid["nz"]], np.int32)
    gd = np.array([grid[k] for k in ("xmin", "ymin", "zmin", "dx", "dy", "dz", "scaling", "water_depth")])
    iset = np.array([settings[k] for k in ("raylov", "gridx", "gridy", "sgref", "sgdic", "sgext", "order",
                                           "sigdep", "material_law")], np.int32)
    npd = len(data["freqs"])
    nsta = len(data["src"])
    freqs, src, raystat, ttime = f(data["freqs"]), f(data["src"]), f(data["raystat"], np.int32), f(data["ttime"])
    shape = (grid["nx"], grid["ny"], grid["nz"])

    def vs_grid(p, q, n):
        sid = np.zeros(shape, np.int32)
        a, b, c = np.zeros(shape), np.zeros(shape), np.zeros(shape)
        orc.orc_kdtree_to_grid(3, n, P(f(p[:n])), P(f(q[:n])), *shape, grid["xmin"], grid["ymin"], grid["zmin"],
                               grid["dx"], grid["dy"], grid["dz"], 1, shape[0], 1, shape[1], 1, shape[2],
                               P(sid), P(a), P(b), P(c))
        return b

    def like(p, q, n, c, mask, pv, pt=None):
        out = np.zeros(4)
        orc.orc_surf_likelihood(P(gi), P(gd), P(iset), settings["dphase"], settings["rho_value"], n,
                                P(f(p[:n])), P(f(q[:n])), npd, P(freqs), nsta, P(src), nsta, P(src), P(raystat),
                                P(ttime), None, data["nrays"], P(f(n0[c])), P(f(n1[c])), P(mask), P(pv), P(pt),
                                P(out))
        return out

    t_total = 0.0
    for k, (c, st) in enumerate(sample_proposals(len(ncells), len(props), nprop)):
        n = int(ncells[c])
        pv = np.zeros((npd, grid["nx"], grid["ny"]))
        p0, q0 = committed_state(init, props, c, st)
        like(p0, q0, n, c, None, pv)          # committed state (untimed)
        p1, q1 = props[st][0][c], props[st][1][c]
        mask = f((vs_grid(p0, q0, n) != vs_grid(p1, q1, n)).any(axis=2).reshape(-1), np.int32)
        pt = np.zeros((npd, nsta, nsta)) if collect is not None else None
        t0 = time.perf_counter()
        out = like(p1, q1, n, c, mask, pv, pt)
        t_total += time.perf_counter() - t0
        if collect is not None:
            collect.append((c, st, pt, pv.copy(), out))
    return nprop / t_total


def sample_proposals(nchains, nsteps, nprop):
    """(chain, step) of the sampled proposals: chains spread over the whole
    batch, steps spread over the whole run."""
    out = []
    for k in range(nprop):
        c = (k * 37 + 5) % nchains
        st = (k * max(1, nsteps // max(nprop, 1))) % nsteps
        out.append((c, st))
    return out


def committed_state(init, props, c, st):
    """Chain c's committed nucleus set before step st (every step commits)."""
    if st == 0:
        return init[0][c], init[1][c]
    return props[st - 1][0][c], props[st - 1][1][c]


def cpu_baseline(grid, settings, data, ncells, init, props, n0, n1, args, collect=None):
    threads = os.cpu_count() or 1
    nprop = args.cpu_sample
    v = cpu_sample(grid, settings, data, ncells, init, props, n0, n1, nprop, threads, collect)
    return {"value": round(v, 4), "unit": "proposal evals/s", "cores": threads, "kind": "port",
            "sample": "%d move proposals of the same workload (one chain each, changed columns only), "
                      "C++ restatement of the reference's Fortran path with OpenMP over columns and periods"
                      % nprop}


def surface_accuracy(grid, settings, data, ncells, init, props, n0, n1, collected):
    """The GPU path on the oracle's sampled proposals (a one-slot context,
    the chain's committed state first): max differences of the travel times
    (paths with data), the phase-velocity maps and -log L."""
    from mctomo_gb300 import SurfaceLikelihood
    lk = SurfaceLikelihood(grid, settings, data, nslots=1, ncell_max=NCELL_MAX)
    rays = np.asarray(data["raystat"]).reshape(len(data["freqs"]), len(data["src"]), len(data["src"])) == 1
    err_t = err_v = err_l = 0.0
    errs = []
    one = np.zeros(1, np.int32)
    for c, st, ept, epv, eout in collected:
        sl = np.zeros(1, np.int32)
        p0, q0 = committed_state(init, props, c, st)
        lk.forward(sl, ncells[c:c + 1], p0[None], q0[None], n0[c:c + 1], n1[c:c + 1])
        lk.commit(one + 1)
        o = lk.forward(sl, ncells[c:c + 1], props[st][0][c:c + 1], props[st][1][c:c + 1], n0[c:c + 1],
                       n1[c:c + 1])
        lk.commit(one)
        pt, pv = lk.phase_time(0)
        e = np.abs(pt - ept)[rays]
        errs.append(e)
        err_t = max(err_t, float(np.max(e)))
        err_v = max(err_v, float(np.max(np.abs(pv - epv))))
        err_l = max(err_l, float(abs(o[0, 0] - eout[0]) / abs(eout[0])))
    lk.close()
    e = np.concatenate(errs) if errs else np.zeros(1)
    return {"proposals_checked": len(collected),
            "sampled_chain_step": [[int(c), int(st)] for c, st, _, _, _ in collected],
            "paths_checked": int(e.size), "max_ttime_err_s": err_t,
            "p99_ttime_err_s": float(np.quantile(e, 0.99)), "frac_paths_within_1e-4_s": float(np.mean(e <= 1e-4)),
            "max_phase_vel_err_kms": err_v, "max_like_rel_err": err_l,
            "reference": "oracle restatement of the reference path, FP64"}


def run_reference(args):
    ws, rank = dist_env()
    if rank != 0:
        return
    grid, settings, data, ncells, init, props, n0, n1 = make_workload(2)
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        cpu_sample(grid, settings, data, ncells, init, props, n0, n1, 1, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_sample(grid, settings, data, ncells, init, props, n0, n1, args.cpu_sample, threads))
    dt = time.perf_counter() - t0
    value = statistics.mean(vals)
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "proposal evals/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, shapes of the configuration)",
            "config": CONFIG,
            "cpu_baseline": {"value": round(value, 4), "unit": "proposal evals/s", "cores": threads, "kind": "port",
                             "sample": "%d move proposals per step, C++ restatement of the reference path"
                                       % args.cpu_sample},
            "e2e": {"value": round(value, 4), "unit": "proposal evals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


BODY_CONFIG = {"workload": "batched 3D body-wave (P and S first arrivals) likelihood: 101x101x51 grid over "
                           "50x50x25 km, 20-800 Voronoi cells/chain, 200 events at 1-20 km depth, 60 surface "
                           "stations, 24,000 picks, solved from the stations (reciprocity)",
               "grid": [101, 101, 51], "events": 200, "stations": 60, "phases": 2}
BODY_SOLVERS = {
    "tiles": ("tile-based fast iterative method on the reference's update", "ttime err<=1e-4 (first order)",
              "f32 local solves on int32 fixed-point times; f64 gridding and misfit"),
    "heap": ("exact heap march: the reference's SFMM step for step", "ttime identical to the reference",
             "f64 updates in the reference's operation order; f64 gridding and misfit"),
}


DROPIN_CONFIG = {"workload": "the reference's body-wave loop with the per-solve drop-in: per proposal, "
                             "kdtree_to_grid (mct_kdtree_to_grid) then one fastMarching3D call "
                             "(mct_fast_marching3d) per station and phase from a pool of host threads, as the "
                             "reference's OpenMP loop over stations; 101x101x51 grid over 50x50x25 km, 200 events, "
                             "60 stations, P and S (120 solves per proposal)",
                 "grid": [101, 101, 51], "events": 200, "stations": 60, "phases": 2}


def run_dropin(args):
    """Configuration 3 through the literal drop-in (src/likelihood_body.F90:
    204-224): each proposal grids the chain's model with mct_kdtree_to_grid
    and makes one mct_fast_marching3d call per station and phase from a pool
    of args.dropin_threads host threads (each thread has its own stream and
    workspace in the library). The oracle runs the same proposals on the
    host cores (the reference's SFMM restated) for the CPU column and the
    accuracy check."""
    import concurrent.futures as cf
    import torch
    from mctomo_gb300 import fast_marching3d, forward, synthetic
    rng = np.random.default_rng(SEED + 1)
    grid, settings, data, ev = synthetic.body_workload(rng)
    settings["order"] = args.order
    nx, ny, nz = grid["nx"], grid["ny"], grid["nz"]
    h = (grid["dx"], grid["dy"], grid["dz"] / grid["scaling"])
    lo3 = (grid["xmin"], grid["ymin"], grid["zmin"] / grid["scaling"])
    rev = np.asarray(data["rev"]); locs = np.ascontiguousarray(ev[:, :3])
    npp = settings["np"]
    lo = np.zeros(3); hi = np.array([50.0, 50.0, 25.0])
    ncell_max = 800
    props = []
    for _ in range(args.warmup + args.steps):
        n = int(rng.integers(20, ncell_max + 1))
        p, q = synthetic.voronoi_model_3d(rng, n, lo, hi, (3.0 / 1.73, 7.5 / 1.73))
        q[:, 0] = q[:, 1] * 1.73
        props.append((n, p, q))
    threads = args.dropin_threads
    solver = None if args.order == 1 else "tiles"

    def proposal(n, p, q):
        _, vp, vs, _ = forward.kdtree_to_grid(p, q, nx, ny, nz, (grid["xmin"], grid["ymin"], grid["zmin"]),
                                              (grid["dx"], grid["dy"], grid["dz"]))
        vels = (vp, vs)
        pt = np.zeros((npp, data["nsrc"], len(rev)))

        def solve(job):
            ph, k = job
            pt[ph, :, k] = fast_marching3d(vels[ph], h, lo3, rev[k], locs, order=args.order, solver=solver)

        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(solve, [(ph, k) for ph in range(npp) for k in range(len(rev))]))
        return pt

    for i in range(args.warmup):
        proposal(*props[i])
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    ms, pts = [], []
    for i in range(args.warmup, args.warmup + args.steps):
        t0 = time.perf_counter()
        pts.append(proposal(*props[i]))
        ms.append((time.perf_counter() - t0) * 1e3)
    cl = clocks.stop()
    value = 1e3 * len(ms) / sum(ms)
    line = {"metric": "proposal evals/s through the per-solve drop-in (fastMarching3D per station and phase "
                      "from %d host threads)" % threads,
            "value": round(value, 4), "unit": "proposal evals/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(sum(ms) / len(ms), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 local solves on int32 fixed-point times (tile solver)" if args.order == 0 else
                     "f64 heap march in the reference's operation order",
            "data": "synthetic (seeded, shapes of the configuration)",
            "config": dict(DROPIN_CONFIG, order=args.order, host_threads=threads),
            "e2e": {"value": round(value, 4), "unit": "proposal evals/s",
                    "h2d_bytes_per_step": int(npp * len(rev) * (nx * ny * nz * 8 + 24 + len(ev) * 24)),
                    "d2h_bytes_per_step": int(npp * len(rev) * len(ev) * 8)},
            "p50_ms": round(float(np.percentile(ms, 50)), 3), "p99_ms": round(float(np.percentile(ms, 99)), 3),
            "gpu_launches": None, "clocks": cl}
    if not args.no_cpu:
        k = args.warmup
        n, p, q = props[k]
        ept, _, dt = body_oracle_proposal(grid, settings, data, ev, n, p, q, np.zeros(npp), np.full(npp, 0.05),
                                          os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": round(1.0 / dt, 4), "unit": "proposal evals/s",
                                "cores": os.cpu_count() or 1, "kind": "reference",
                                "sample": "1 proposal: kd-tree gridding + 120 fastMarching3D solves (the "
                                          "reference's SFMM restated bit-exactly) on a thread pool over all host "
                                          "cores, misfit"}
        rays = np.asarray(data["raystat"]).reshape(ept.shape) == 1
        e = np.abs(pts[0] - ept)[rays]
        line["accuracy"] = {"proposals_checked": 1, "times_checked": int(e.size), "max_ttime_err_s": float(e.max()),
                            "p99_ttime_err_s": float(np.quantile(e, 0.99)),
                            "frac_times_within_1e-4_s": float(np.mean(e <= 1e-4)),
                            "reference": "oracle restatement of the reference's fastMarching3D (FP64)"}
    print(json.dumps(line), flush=True)


def run_body(args):
    """The body-wave configuration: every step is one full proposal per chain
    (gridding, 120 3D solves, misfit) through the host API."""
    import torch
    from mctomo_gb300 import BodyLikelihood, synthetic
    ws, rank = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    dev = torch.device("cuda")
    nch = args.chains
    rng = np.random.default_rng(SEED + 1)
    grid, settings, data, ev = synthetic.body_workload(rng)
    settings["order"] = args.order
    solver = args.solver or ("heap" if args.order == 1 else "tiles")
    settings["solver"] = {"tiles": 0x10, "heap": 0x20}[solver]
    settings["dynamic"] = 1 if args.dynamic else 0
    lo = np.zeros(3); hi = np.array([50.0, 50.0, 25.0])
    ncell_max = 800
    props = []
    for _ in range(args.warmup + args.steps):
        ncells = rng.integers(20, ncell_max + 1, nch).astype(np.int32)
        pts = np.zeros((nch, ncell_max, 3)); par = np.zeros((nch, ncell_max, 3))
        for c in range(nch):
            p, q = synthetic.voronoi_model_3d(rng, int(ncells[c]), lo, hi, (3.0 / 1.73, 7.5 / 1.73))
            q[:, 0] = q[:, 1] * 1.73
            pts[c, :ncells[c]] = p; par[c, :ncells[c]] = q
        props.append((ncells, pts, par))
    locs = np.repeat(ev[None], nch, 0)
    n0 = np.zeros((nch, 2)); n1 = np.full((nch, 2), 0.05)
    lk = BodyLikelihood(grid, settings, data, nslots=nch, ncell_max=ncell_max)
    for i in range(args.warmup):
        lk.forward(*props[i], locs, n0, n1)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    ms = []
    for i in range(args.warmup, args.warmup + args.steps):
        t0 = time.perf_counter()
        out = lk.forward(*props[i], locs, n0, n1)
        ms.append((time.perf_counter() - t0) * 1e3)
    cl = clocks.stop()
    value, total = job_rate(nch * args.steps, sum(ms), ws, dev)
    h2d = nch * ncell_max * 3 * 8 * 2 + nch * 4 + nch * len(ev) * 4 * 8 + 2 * nch * 2 * 8
    # the plain drop-in: one chain per call
    one = BodyLikelihood(grid, settings, data, nslots=1, ncell_max=ncell_max)
    ncells0, pts0, par0 = props[0]
    one.forward(ncells0[:1], pts0[:1], par0[:1], locs[:1], n0[:1], n1[:1])
    pms = []
    for i in range(2):
        nc, pp, qq = props[(i + 1) % len(props)]
        t0 = time.perf_counter()
        one.forward(nc[:1], pp[:1], qq[:1], locs[:1], n0[:1], n1[:1])
        pms.append((time.perf_counter() - t0) * 1e3)
    one.close()
    location = body_location_steps(lk, grid, settings, data, ev, locs, n0, n1, args) if args.dynamic else None
    desc, err, dtype = BODY_SOLVERS[solver]
    from mctomo_gb300 import lib as _mlib
    # the tile solver's tuned configuration (shape index * 4 + sweeps index)
    tile_cfg = int(_mlib().mct_eik3_tile_config(-2, grid["nx"], grid["ny"], grid["nz"], args.order))
    line = {"metric": "body-wave forward evals/s, 1 GB300, " + err, "value": round(value, 4),
            "unit": "proposal evals/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(total / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype,
            "data": "synthetic (seeded, shapes of the configuration)",
            "config": dict(BODY_CONFIG, chains=nch, order=args.order, eikonal=desc,
                           tile_config=(tile_cfg if solver == "tiles" else None)),
            "e2e": {"value": round(value, 4), "unit": "proposal evals/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": nch * 4 * 8},
            "note": "host API only (value = e2e): the body context has no device-pointer forward",
            "batched_latency_ms": {"p50": round(float(np.percentile(ms, 50)), 3),
                                   "p99": round(float(np.percentile(ms, 99)), 3)},
            "plain": {"value": round(1e3 / float(np.mean(pms)), 4), "unit": "proposal evals/s",
                      "p50_ms": round(float(np.percentile(pms, 50)), 3),
                      "p99_ms": round(float(np.percentile(pms, 99)), 3)},
            "clocks": cl, "valid_models": int((out[:, 3] == 0).sum())}
    if location is not None:
        line["location"] = location
    if rank == 0:
        chains = sorted({0, nch // 3, (2 * nch) // 3})[:args.body_sample]
        try:
            cpu, acc = body_cpu_and_accuracy(lk, grid, settings, data, ev, props[0], locs, n0, n1, chains,
                                             not args.no_cpu)
            if cpu is not None:
                line["cpu_baseline"] = cpu
            line["accuracy"] = acc
        except Exception as e:   # the throughput line stands without it
            line["accuracy"] = {"error": "%s: %s" % (type(e).__name__, e)}
        print(json.dumps(line), flush=True)
    lk.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def body_location_steps(lk, grid, settings, data, ev, locs, n0, n1, args):
    """Location steps on the stored fields (settings dynamic = 1): the last
    forward's models are committed, then every step proposes new locations
    for all events of every chain (Gaussian, 0.2 km) and evaluates them
    through the host API; the CPU column is the oracle's read-out of the
    same 120 fields per chain (OpenMP over phases and stations) and the
    misfit, for one chain."""
    nch = locs.shape[0]
    lk.commit(np.ones(nch, np.int32))
    rng = np.random.default_rng(SEED + 9)
    ext = np.array([grid["dx"] * (grid["nx"] - 1), grid["dy"] * (grid["ny"] - 1), grid["dz"] * (grid["nz"] - 1)])
    props = []
    for _ in range(args.warmup + args.steps):
        p = locs.copy()
        p[:, :, :3] = np.clip(p[:, :, :3] + rng.normal(0, 0.2, p[:, :, :3].shape), 0.0, ext)
        props.append(p)
    for i in range(args.warmup):
        lk.location_likelihood(props[i], n0, n1)
    ms = []
    for i in range(args.warmup, args.warmup + args.steps):
        t0 = time.perf_counter()
        out = lk.location_likelihood(props[i], n0, n1)
        ms.append((time.perf_counter() - t0) * 1e3)
    res = {"value": round(nch * len(ms) / (sum(ms) / 1e3), 2), "unit": "location steps/s (chains x steps)",
           "ms_per_step": round(float(np.mean(ms)), 4), "p50_ms": round(float(np.percentile(ms, 50)), 4),
           "p99_ms": round(float(np.percentile(ms, 99)), 4), "valid": int((out[:, 3] == 0).sum()),
           "reads_per_step": int(nch * settings["np"] * data["nsrc"] * len(data["rev"]))}
    if not args.no_cpu:
        import oracle
        orc = oracle.load()
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        npp, nsrc, nrev = settings["np"], data["nsrc"], len(data["rev"])
        fields = rng.uniform(0.0, 20.0, (npp, nrev, grid["nx"], grid["ny"], grid["nz"]))
        ev0 = np.ascontiguousarray(props[-1][0])
        times = np.zeros((npp, nsrc, nrev))
        reps = 5
        t0 = time.perf_counter()
        for _ in range(reps):
            orc.orc_location_times(grid["nx"], grid["ny"], grid["nz"], grid["xmin"], grid["ymin"], grid["zmin"],
                                   grid["dx"], grid["dy"], grid["dz"], grid["scaling"], npp, nsrc, nrev, P(fields),
                                   P(ev0), P(times))
            body_location_cpu_misfit(orc, settings, data, ev0, times, n0[0], n1[0])
        dt = (time.perf_counter() - t0) / reps
        res["cpu_baseline"] = {"value": round(1.0 / dt, 2), "unit": "location steps/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": "%d location steps of one chain: the oracle's Interpolate3d "
                                                         "read-out of its %d stored fields (OpenMP) and misfit"
                                                         % (reps, npp * nrev)}
    return res


def body_location_cpu_misfit(orc, settings, data, ev, pt, n0, n1):
    """The oracle's misfit of a location step (sigma = n0 * time + n1)."""
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    npp, nsrc, nrev = pt.shape
    npairs = nsrc * nrev
    dtt = np.zeros((npp, 3, npairs))
    dtt[:, 0] = np.asarray(data["ttime"]).reshape(npp, npairs)
    rs = np.zeros((npp, 2, npairs), np.int32); rs[:, 0] = np.asarray(data["raystat"]).reshape(npp, npairs)
    sig = np.zeros((npp, npairs)); out = np.zeros(3)
    ptf = np.ascontiguousarray(pt.reshape(npp, npairs))
    orc.orc_body_misfit(nsrc, nrev, npp, P(ptf), P(np.ascontiguousarray(ev[:, 3])), P(np.ascontiguousarray(dtt)),
                        P(np.ascontiguousarray(rs)), P(ptf), 1, P(np.ascontiguousarray(n0)),
                        P(np.ascontiguousarray(n1)), data["nrays"], P(sig), P(out))
    return out


def body_oracle_proposal(grid, settings, data, ev, n, pts, par, n0, n1, threads):
    """The oracle's restatement of the reference's body path for one chain's
    proposal: kd-tree gridding, then fastMarching3D from each station for P
    and S (the reference's OpenMP loop over stations, here a thread pool),
    then the misfit reduction. Returns (phase times (np, nsrc, nrev), misfit
    out, seconds)."""
    import concurrent.futures as cf
    import oracle
    orc = oracle.load()
    P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    nx, ny, nz = grid["nx"], grid["ny"], grid["nz"]
    shp = (nx, ny, nz)
    rev = np.asarray(data["rev"])
    locs = np.ascontiguousarray(ev[:, :3])
    dzs, zms = grid["dz"] / grid["scaling"], grid["zmin"] / grid["scaling"]
    npp = settings["np"]
    t0 = time.perf_counter()
    sid = np.zeros(shp, np.int32); vp = np.zeros(shp); vs = np.zeros(shp); rho = np.zeros(shp)
    orc.orc_kdtree_to_grid(3, n, P(np.ascontiguousarray(pts[:n])), P(np.ascontiguousarray(par[:n])), nx, ny,
                           nz, grid["xmin"], grid["ymin"], grid["zmin"], grid["dx"], grid["dy"], grid["dz"], 1, nx, 1,
                           ny, 1, nz, P(sid), P(vp), P(vs), P(rho))
    jobs = [(p, k) for p in range(npp) for k in range(len(rev))]
    vels = [vp, vs]
    pt = np.zeros((npp, data["nsrc"], len(rev)))

    def solve(job):
        p, k = job
        tt = np.zeros(data["nsrc"])
        orc.orc_fast_marching3d(nx, ny, nz, grid["dx"], grid["dy"], dzs, grid["xmin"], grid["ymin"], zms,
                                P(vels[p]), P(np.ascontiguousarray(rev[k])), P(locs), data["nsrc"],
                                settings["order"], P(tt), None)
        pt[p, :, k] = tt

    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(solve, jobs))
    # the misfit with origin times (src/likelihood_body.F90:284-333)
    nsrc, nrev = data["nsrc"], len(rev)
    npairs = nsrc * nrev
    dtt = np.zeros((npp, 3, npairs))
    dtt[:, 0] = np.asarray(data["ttime"]).reshape(npp, npairs)
    dtt[:, 1] = np.asarray(data["sigma"]).reshape(npp, npairs)
    rs = np.zeros((npp, 2, npairs), np.int32); rs[:, 0] = np.asarray(data["raystat"]).reshape(npp, npairs)
    sig = np.zeros((npp, npairs)); out = np.zeros(3)
    ptf = np.ascontiguousarray(pt.reshape(npp, npairs))
    orc.orc_body_misfit(nsrc, nrev, npp, P(ptf), P(np.ascontiguousarray(ev[:, 3])), P(np.ascontiguousarray(dtt)),
                        P(np.ascontiguousarray(rs)), P(ptf), settings["sigdep"], P(np.ascontiguousarray(n0)),
                        P(np.ascontiguousarray(n1)), data["nrays"], P(sig), P(out))
    return pt, out, time.perf_counter() - t0


def body_cpu_and_accuracy(lk, grid, settings, data, ev, prop, locs, n0, n1, chains, with_cpu):
    """The oracle on whole proposals (every one of the 120 solves) of the
    given chains of one step: the first one timed as the CPU baseline; the
    GPU context's travel times and -log L for the same proposals (one more
    forward of that step) compared with it."""
    threads = os.cpu_count() or 1
    ncells, pts, par = prop
    out_gpu = lk.forward(ncells, pts, par, locs, n0, n1)
    errs, err_l, cpu = [], 0.0, None
    for c in chains:
        ept, eout, dt = body_oracle_proposal(grid, settings, data, ev, int(ncells[c]), pts[c], par[c], n0[c], n1[c],
                                             threads)
        if cpu is None:
            cpu = {"value": round(1.0 / dt, 4), "unit": "proposal evals/s", "cores": threads, "kind": "reference",
                   "sample": "1 proposal (one chain): kd-tree gridding + 120 fastMarching3D solves (the reference's "
                             "own C++ SFMM as restated bit-exactly) on a thread pool over all host cores, misfit"}
        pt, _ = lk.phase_time(c)
        rays = np.asarray(data["raystat"]).reshape(pt.shape) == 1
        errs.append(np.abs(pt - ept)[rays])
        err_l = max(err_l, float(abs(out_gpu[c, 0] - eout[0]) / abs(eout[0])))
    e = np.concatenate(errs)
    acc = {"proposals_checked": len(chains), "sampled_chains": [int(c) for c in chains],
           "times_checked": int(e.size), "max_ttime_err_s": float(e.max()),
           "p99_ttime_err_s": float(np.quantile(e, 0.99)), "frac_times_within_1e-4_s": float(np.mean(e <= 1e-4)),
           "max_like_rel_err": err_l,
           "reference": "oracle restatement of the reference's fastMarching3D (FP64, pinned bit-for-bit to the "
                        "compiled reference) + misfit"}
    return (cpu if with_cpu else None), acc


# FP64 operations (add, sub, mul, div, sqrt) of one layer iteration of the
# period equation, counted from the source (surfdisp96.f:1119-1217 with var
# 1220-1337, dnka 1370-1414, normc 1341-1366 for Rayleigh; dltar1
# 1056-1115 for Love), propagating case; sin / cos / exp are counted
# separately (5 per Rayleigh layer, 2 per Love layer). Rayleigh: layer
# set-up 16 (3 div, 2 sqrt) + var 14 (2 div) + dnka 78 (4 div) + 5x5
# matrix-vector product 50 + normalisation 5 (div) = 163. Love: 20 (4 div,
# 1 sqrt).
DISP_OPS_PER_LAYER = {2: 163, 1: 20}
# FP64 peak: ncu reports sm__sass_thread_inst_executed_op_dfma_pred_on
# .sum.peak_sustained = 304 DFMA per cycle on this GPU (2 per SM), i.e.
# 304 x 2 flop x 2.07 GHz (maximum SM clock) = 1.259 TFLOP/s. It is the
# device's rated issue rate, not a timed measurement.
FP64_PEAK_TFLOPS = 304 * 2 * 2.07e9 / 1e12
DISP_CONFIG = {"workload": "dispersion-precision study: 262,144 independent layered columns (12-40 layers, "
                           "thickness U[0.05,0.5] km, Vs U[0.2,3.5] km/s with a 10% low-velocity-layer chance, "
                           "Vp = 1.73 Vs, Gardner density), 60 periods 0.2-20 s, Rayleigh and Love, fundamental "
                           "and first overtone, phase and group",
               "periods": 60, "modes": 2, "waves": ["Rayleigh", "Love"]}


def run_disp(args):
    """The dispersion-precision study: every step computes all columns'
    phase and group curves for both wave types and both modes with one
    variant; the FP64 variant and the FP32-bracketing variant are both timed
    on the device, and a seeded sample of columns is compared with the
    oracle (the surfdisp96 restatement), separately for columns with
    low-velocity layers (which the reference's surfmodes routes to GRT)."""
    import torch
    from mctomo_gb300 import _lib, forward, synthetic
    L = _lib.lib()
    dev = torch.device("cuda")
    rng = np.random.default_rng(SEED + 3)
    ncol = args.columns
    nl, thk, vp, vs, rho = synthetic.layered_columns(rng, ncol, nl_range=(12, 40), lvl_prob=0.1)
    periods = np.geomspace(0.2, 20.0, 60)
    nl_max = thk.shape[1]
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in
         dict(nl=nl, thk=thk, vp=vp, vs=vs, rho=rho, per=periods).items()}
    cp = torch.zeros((ncol, 2, 60), dtype=torch.float64, device=dev)
    cg = torch.zeros_like(cp)
    ierr = torch.zeros(ncol, dtype=torch.int32, device=dev)
    cnt = torch.zeros(2, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()

    # Rayleigh over all columns; Love over the first --love-cols columns (all
    # by default)
    love_cols = min(ncol, args.love_cols) if args.love_cols else ncol
    chunk = ncol          # one launch per wave: every column's warp runs at once

    def study(precision):
        for iwave, nc in ((2, ncol), (1, love_cols)):
            for c0 in range(0, nc, chunk):
                n = min(chunk, nc - c0)
                rc = L.mct_surfdisp_batch_device(n, nl_max, d["nl"][c0:].data_ptr(), d["thk"][c0:].data_ptr(),
                                                 d["vp"][c0:].data_ptr(), d["vs"][c0:].data_ptr(),
                                                 d["rho"][c0:].data_ptr(), 60, d["per"].data_ptr(), iwave, 2, 1,
                                                 0.001, 1, precision, cp[c0:].data_ptr(), cg[c0:].data_ptr(),
                                                 ierr[c0:].data_ptr(), cnt.data_ptr(), stream.cuda_stream)
                _lib.check("mct_surfdisp_batch_device", rc)

    res = {}
    clocks = Clocks(0)
    for precision in (1, 0):
        for _ in range(args.warmup):
            study(precision)
        torch.cuda.synchronize()
        if precision == 1:
            clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            study(precision)
        e1.record(stream)
        torch.cuda.synchronize()
        if precision == 1:
            cl = clocks.stop()
        ms = e0.elapsed_time(e1) / args.steps
        res[precision] = (ms, (ncol + love_cols) * 2 / (ms / 1e3))
    # end to end through the host API (column arrays in, curves out), FP32-bracketing variant
    t0 = time.perf_counter()
    for iwave, nc in ((2, ncol), (1, love_cols)):
        for c0 in range(0, nc, chunk):
            sl = slice(c0, min(nc, c0 + chunk))
            forward.surfdisp_batch(nl[sl], thk[sl], vp[sl], vs[sl], rho[sl], periods, iwave, 1, 0.001, mode=2,
                                   multimode=True, precision=1)
    e2e_s = time.perf_counter() - t0
    acc = disp_oracle_sample(nl, thk, vp, vs, rho, periods, args)
    value = res[1][1]
    # Roofline of the FP64 variant, whose evaluations are the reference's own:
    # algorithmic FP64 operations = the oracle's layer-evaluations x the
    # operations of one layer of the period equation (see DISP_OPS_PER_LAYER)
    lev = acc.pop("oracle_layer_evals_per_column")
    ops = DISP_OPS_PER_LAYER[2] * lev[2] * ncol + DISP_OPS_PER_LAYER[1] * lev[1] * love_cols
    achieved = ops / (res[0][0] / 1e3) / 1e12
    roofline = {"kernel": "surfdisp_kernel, FP64 variant", "bound": "fp64", "achieved": round(achieved, 4),
                "peak": round(FP64_PEAK_TFLOPS, 4),
                "peak_kind": "rated (ncu: 2 DFMA/cycle/SM x 152 SMs x 2.07 GHz); MEASURED_PEAKS.json has no FP64 figure",
                "unit": "TFLOP/s", "frac": round(achieved / FP64_PEAK_TFLOPS, 4), "traffic": None,
                "algorithmic_fp64_ops_per_step": round(ops), "ops_per_layer": DISP_OPS_PER_LAYER,
                "transcendentals_per_layer": {"rayleigh": 5, "love": 2}}
    line = {"metric": "dispersion curves/s (column x wave x mode, phase + group), 1 GB300, phase err<=1e-5 km/s",
            "value": round(value, 2), "unit": "curves/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(res[1][0], 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 bracketing confirmed in f64, f64 polish (precision 1); f64 throughout (precision 0)",
            "data": "synthetic (seeded, shapes of the configuration)",
            "config": dict(DISP_CONFIG, rayleigh_columns=ncol, love_columns=love_cols),
            "variants": {"fp32_bracketing_fp64_polish": {"ms_per_step": round(res[1][0], 3),
                                                         "curves_per_s": round(res[1][1], 2)},
                         "fp64": {"ms_per_step": round(res[0][0], 3), "curves_per_s": round(res[0][1], 2)}},
            "e2e": {"value": round((ncol + love_cols) * 2 / e2e_s, 2), "unit": "curves/s",
                    "h2d_bytes_per_step": int(4 * 4 * ncol * nl_max + 4 * ncol + 60 * 8) * 2,
                    "d2h_bytes_per_step": int(2 * ncol * 2 * 60 * 8 + 4 * ncol) * 2},
            "accuracy": acc, "clocks": cl, "roofline": roofline, "gpu_launches": 4 * args.steps}
    if not args.no_cpu:
        line["cpu_baseline"] = acc.pop("cpu_baseline")
    else:
        acc.pop("cpu_baseline", None)
    print(json.dumps(line), flush=True)


def disp_oracle_sample(nl, thk, vp, vs, rho, periods, args):
    """The oracle (surfdisp96 / surfdisp_mmodes restated) on a seeded sample
    of columns, both waves, both modes, phase and group, on a thread pool
    over all host cores; max phase and group differences of both GPU
    variants on that sample, columns with low-velocity layers apart."""
    import concurrent.futures as cf
    import oracle
    from mctomo_gb300 import forward
    orc = oracle.load()
    P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rng = np.random.default_rng(SEED + 4)
    idx = np.sort(rng.choice(min(len(nl), args.love_cols or len(nl)), args.disp_sample, replace=False))
    cols = [tuple(np.ascontiguousarray(x[c, :nl[c]]) for x in (thk, vp, vs, rho)) for c in idx]
    lvl = np.array([bool(np.any(np.diff(vs[c, :nl[c]]) < 0)) for c in idx])
    threads = os.cpu_count() or 1
    out = {}
    t0 = time.perf_counter()
    for iwave in (2, 1):
        def one(k):
            o1 = np.zeros(120); o2 = np.zeros(120); n = np.zeros(1, np.int64)
            e = orc.orc_surfdisp_mmodes(*[P(x) for x in cols[k]], int(len(cols[k][0])), iwave, 2, 1, 60,
                                        P(periods), 0.001, P(o1), P(o2), P(n))
            return e, o1.reshape(2, 60), o2.reshape(2, 60), int(n[0])
        with cf.ThreadPoolExecutor(threads) as ex:
            out[iwave] = list(ex.map(one, range(len(idx))))
    cpu_s = time.perf_counter() - t0
    acc = {"columns_sampled": int(len(idx)), "lvl_columns_sampled": int(lvl.sum())}
    # the reference's own FP64 work, counted by the oracle: evaluations x layer
    # iterations per evaluation (nl - llw; llw = 2 under a water layer), mean
    # per column of the sample, per wave type
    layers = np.array([len(c[0]) - (2 if c[2][0] <= 0 else 1) for c in cols])
    acc["oracle_layer_evals_per_column"] = {
        w: float(np.mean([out[w][k][3] * layers[k] for k in range(len(idx))])) for w in (2, 1)}
    for precision, name in ((1, "fp32_bracketing_fp64_polish"), (0, "fp64")):
        worst = {"plain": [0.0, 0.0], "lvl": [0.0, 0.0]}
        agree = 0
        for iwave in (2, 1):
            cp, cg, ierr, _ = forward.surfdisp_batch(nl[idx], thk[idx], vp[idx], vs[idx], rho[idx], periods, iwave,
                                                     1, 0.001, mode=2, multimode=True, precision=precision)
            for k in range(len(idx)):
                e, ecp, ecg, _ = out[iwave][k]
                agree += int(e == ierr[k])
                good = (ecp > 0) & (cp[k] > 0)
                key = "lvl" if lvl[k] else "plain"
                if good.any():
                    worst[key][0] = max(worst[key][0], float(np.max(np.abs(cp[k][good] - ecp[good]))))
                    worst[key][1] = max(worst[key][1], float(np.max(np.abs(cg[k][good] - ecg[good]))))
        acc[name] = {"max_phase_err_kms": worst["plain"][0], "max_group_err_kms": worst["plain"][1],
                     "lvl_max_phase_err_kms": worst["lvl"][0], "lvl_max_group_err_kms": worst["lvl"][1],
                     "ierr_agreement": round(agree / (2 * len(idx)), 4)}
    acc["cpu_baseline"] = {"value": round(len(idx) * 4 / cpu_s, 2), "unit": "curves/s", "cores": threads,
                           "kind": "port", "sample": "%d seeded columns of the study, both waves, modes 1-2, phase "
                                                     "and group, surfdisp restatement (oracle)" % len(idx)}
    return acc


TT2D_CONFIG = {"workload": "plain 2D travel-time likelihood (the 2D code's path): 51x51 grid over 10x10 km, "
                           "16 stations on a square perimeter, every station a source to the others (240 times), "
                           "Voronoi velocity models (4-100 cells, 2-4 km/s), fm2d with the 2D example's settings "
                           "(gridx=gridy=1, sgref=1, sgdic=5, sgext=10, order=1), FP64 (reference order)",
               "grid": [51, 51], "stations": 16, "times": 240}


# FP64 operations per secular evaluation of the generalized R/T search as the
# kernel executes them: DADD + DMUL + 2 x DFMA thread instructions (ncu
# counters) over the evaluations of `bench.py --case grt --case-columns 20`
# (Rayleigh, then --case-order 0 for Love), search logic included
GRT_FP64_FLOPS_PER_EVAL = {1: (21567665 + 22925835 + 2 * 31357386) / 4276,
                           0: (24931182 + 46682971 + 2 * 149068957) / 13014}
GRT_CONFIG = {"workload": "generalized R/T fundamental-mode dispersion (the reference's single-mode surfmodes path "
                         "for low-velocity-layer columns): layered columns drawn as the dispersion study's (12-40 "
                         "layers, h U[0.05,0.5] km, Vs U[0.2,3.5] km/s with a 10% low-velocity-layer chance, "
                         "Vp = 1.73 Vs, rho = 1.74 Vp^0.25), routed as surfmodes routes them (setup_grt's nlvls1 > "
                         "0), Rayleigh and Love, phase and group, 60 periods 0.2-20 s (ascending), tol 1e-6, "
                         "dc 1e-3",
              "periods": 60, "inputs": "larger than L2 (per-lane trial-velocity scratch of GBs)"}


def run_grt(args):
    """Generalized R/T fundamental-mode dispersion curves of the columns that
    surfmodes routes to RayleighModes / LoveModes (surfmodes.f90:39-108,
    185-303): device path timed with CUDA events, host-buffer path end to
    end, the oracle on a sample of the same columns on all host cores."""
    import torch
    from mctomo_gb300 import _lib, forward, synthetic
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    L = _lib.lib()
    rng = np.random.default_rng(SEED + 7)
    nl, thk, vp, vs, rho = synthetic.layered_columns(rng, args.grt_cols, nl_range=(12, 40), lvl_prob=0.1)
    thk, vp, vs, rho = (np.ascontiguousarray(x, np.float64) for x in (thk, vp, vs, rho))
    periods = np.geomspace(0.2, 20.0, 60)
    freqs = np.ascontiguousarray(1.0 / periods)
    waves = {}
    for mt in (1, 0):
        route = forward.surfmodes_route(nl, vp, vs, mt)
        sel = np.where(route == 1)[0]
        waves[mt] = sel
    streams = {1: torch.cuda.Stream(dev), 0: torch.cuda.Stream(dev)}
    dbuf = {}
    for mt, sel in waves.items():
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        dbuf[mt] = dict(nl=t(nl[sel].astype(np.int32)), thk=t(thk[sel]), vp=t(vp[sel]), vs=t(vs[sel]),
                        rho=t(rho[sel]), ph=torch.zeros((len(sel), 60), dtype=torch.float64, device=dev),
                        gr=torch.zeros((len(sel), 60), dtype=torch.float64, device=dev),
                        ierr=torch.zeros(len(sel), dtype=torch.int32, device=dev),
                        cnt=torch.zeros(1, dtype=torch.int64, device=dev))
    d_f = torch.from_numpy(freqs).to(dev)
    paras = {mt: forward.modes_para(mt, 1, tol=1e-6, dc=1e-3) for mt in (1, 0)}
    nl_max = thk.shape[1]

    def launch(mt, ncols):
        b = dbuf[mt]
        rc = L.mct_grt_batch_device(ncols, nl_max, b["nl"].data_ptr(), b["thk"].data_ptr(),
                                    b["vp"].data_ptr(), b["vs"].data_ptr(), b["rho"].data_ptr(), 60,
                                    d_f.data_ptr(), ctypes.byref(paras[mt]), b["ph"].data_ptr(),
                                    b["gr"].data_ptr(), b["ierr"].data_ptr(), b["cnt"].data_ptr(),
                                    ctypes.c_void_p(streams[mt].cuda_stream))
        _lib.check("mct_grt_batch_device", rc)

    # warm-up: the kernels' first launches on a few columns of each wave
    for _ in range(args.warmup):
        for mt in (1, 0):
            launch(mt, min(64, len(waves[mt])))
    torch.cuda.synchronize()
    for mt in (1, 0):
        dbuf[mt]["cnt"].zero_()
    torch.cuda.synchronize()
    # the two wave types run on their own streams, side by side
    clocks = Clocks(0)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    done0 = torch.cuda.Event()
    s1, s0 = streams[1], streams[0]
    e0.record(s1)
    s0.wait_event(e0)
    for _ in range(args.steps):
        launch(1, len(waves[1]))
        launch(0, len(waves[0]))
    done0.record(s0)
    s1.wait_event(done0)
    e1.record(s1)
    torch.cuda.synchronize()
    cl = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    curves = sum(len(v) for v in waves.values())
    value = curves / (ms / 1e3)
    evals = {mt: int(dbuf[mt]["cnt"].item()) // args.steps for mt in (1, 0)}
    # end to end through the host API, one host thread per wave type (each
    # gets its own stream in the library)
    host = {}

    def host_call(mt):
        sel = waves[mt]
        host[mt] = forward.grt_batch(nl[sel], thk[sel], vp[sel], vs[sel], rho[sel], freqs, paras[mt])
    t0 = time.perf_counter()
    ths = [threading.Thread(target=host_call, args=(mt,)) for mt in (1, 0)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    e2e_s = time.perf_counter() - t0
    lay_b = sum(int(len(v)) * nl_max * 8 * 4 + int(len(v)) * 4 for v in waves.values()) + 60 * 8
    out_b = sum(int(len(v)) * (2 * 60 * 8 + 4) for v in waves.values())
    acc, cpu = grt_oracle_sample(nl, thk, vp, vs, rho, freqs, waves, host, args)
    line = {"metric": "generalized R/T dispersion curves/s (low-velocity-layer columns, fundamental mode, phase + "
                      "group, Rayleigh and Love), 1 GB300",
            "value": round(value, 2), "unit": "curves/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 (complex FP64, no fused multiply-add, the reference's operation order)",
            "data": "synthetic (seeded, shapes of the dispersion study)",
            "config": dict(GRT_CONFIG, columns=int(args.grt_cols), rayleigh_columns=int(len(waves[1])),
                           love_columns=int(len(waves[0]))),
            "secular_evaluations_per_step": evals,
            "secular_evaluations_per_s": round(sum(evals.values()) / (ms / 1e3)),
            "e2e": {"value": round(curves / e2e_s, 2), "unit": "curves/s", "h2d_bytes_per_step": int(lay_b),
                    "d2h_bytes_per_step": int(out_b)},
            "accuracy": acc, "clocks": cl, "roofline": grt_roofline(evals, ms),
            "gpu_launches": args.steps * 2 * 6,
            "timing": "the two wave types on two streams; warm-up launches on 64 columns of each"}
    if not args.no_cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


def grt_roofline(evals, ms):
    """FP64 roofline of the generalized R/T step: the executed FP64
    operations per secular evaluation (ncu) times the evaluations, over the
    step's time, against the FP64 peak."""
    flops = sum(GRT_FP64_FLOPS_PER_EVAL[mt] * evals[mt] for mt in (1, 0))
    achieved = flops / (ms / 1e3) / 1e12
    return {"kernel": "grt_kernel (Rayleigh and Love on two streams)", "bound": "fp64",
            "achieved": round(achieved, 4), "peak": round(FP64_PEAK_TFLOPS, 4),
            "peak_kind": "rated (2 DFMA/cycle/SM x 152 SMs x 2.07 GHz); MEASURED_PEAKS.json has no FP64 figure",
            "unit": "TFLOP/s", "frac": round(achieved / FP64_PEAK_TFLOPS, 4), "traffic": None,
            "fp64_flops_per_evaluation": {"rayleigh": round(GRT_FP64_FLOPS_PER_EVAL[1]),
                                          "love": round(GRT_FP64_FLOPS_PER_EVAL[0])},
            "limiter": "latency of dependent FP64 chains per lane (ncu: dominant stall 'wait'); lanes in flight"}


def grt_oracle_sample(nl, thk, vp, vs, rho, freqs, waves, host, args):
    """The oracle (orc_grt_modes, the reference's RayleighModes / LoveModes
    restated) on the first args.grt_sample routed columns of each wave, on a
    thread pool over all host cores; agreement of the GPU's curves there."""
    import concurrent.futures as cf
    import oracle
    orc = oracle.load()
    P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    threads = os.cpu_count() or 1
    acc = {}
    t0 = time.perf_counter()
    res = {}
    for mt in (1, 0):
        sel = waves[mt][:args.grt_sample]

        def one(c, mt=mt):
            n = int(nl[c])
            a = [np.ascontiguousarray(x[c, :n]) for x in (thk, vp, vs, rho)]
            ph, gr, ne = np.zeros(60), np.zeros(60), np.zeros(1, np.int64)
            e = orc.orc_grt_modes(n, P(a[0]), P(a[1]), P(a[2]), P(a[3]), 60, P(freqs), mt, 1, 1e-6, 1e-5,
                                  float(np.float32(1e-3)), float(np.float32(5e-3)), 1e-3, 1e-3, 1e-3, P(ph), P(gr),
                                  P(ne))
            return e, ph, gr, int(ne[0])
        with cf.ThreadPoolExecutor(threads) as ex:
            res[mt] = list(ex.map(one, sel))
    cpu_s = time.perf_counter() - t0
    ncurves = 0
    for mt, name in ((1, "rayleigh"), (0, "love")):
        ph, gr, ierr, _ = host[mt]
        same = tot = ierr_diff = 0
        worst = 0.0
        for k, (e, eph, egr, _) in enumerate(res[mt]):
            ncurves += 1
            ierr_diff += int(ierr[k] != e)
            d = np.maximum(np.abs(ph[k] - eph), np.abs(gr[k] - egr))
            same += int(np.sum(d <= 1e-9)); tot += d.size
            worst = max(worst, float(np.max(d)))
        acc[name] = {"columns_checked": len(res[mt]), "ierr_mismatches": ierr_diff,
                     "frac_within_1e-9_kms": round(same / max(tot, 1), 5), "max_abs_diff_kms": worst}
    acc["reference"] = "oracle restatement of RayleighModes / LoveModes (FP64)"
    cpu = {"value": round(ncurves / cpu_s, 3), "unit": "curves/s", "cores": threads, "kind": "port",
           "sample": "%d Rayleigh + %d Love routed columns of the same workload, phase + group, 60 periods, "
                     "oracle restatement on a thread pool" % (len(res[1]), len(res[0]))}
    return acc, cpu


def run_tt2d(args):
    """The plain 2D configuration: every step is one value-change proposal
    per chain through the host API (2D gridding, 16 fm2d solves, misfit),
    committed; the plain drop-in is one chain per call."""
    import torch
    from mctomo_gb300 import TravelTime2DLikelihood, synthetic
    rng = np.random.default_rng(SEED + 5)
    grid, settings, data = synthetic.tt2d_workload(rng)
    nch = args.chains2d
    ncells, pts, par = synthetic.tt2d_chain_models(rng, nch, 100, grid)
    props = []
    for _ in range(args.warmup + args.steps):
        q = par.copy()
        for c in range(nch):
            i = rng.integers(ncells[c])
            q[c, i, 0] = np.clip(q[c, i, 0] + rng.normal(0, 0.1), 2.0, 4.0)
        props.append(q)
    n0 = np.zeros((nch, 2)); n1 = np.full((nch, 2), 0.05)
    lk = TravelTime2DLikelihood(grid, settings, data, nslots=nch, ncell_max=100)
    for i in range(args.warmup):
        lk.forward(ncells, pts, props[i], n0, n1)
        lk.commit(np.ones(nch, np.int32))
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    ms = []
    for i in range(args.warmup, args.warmup + args.steps):
        t0 = time.perf_counter()
        out = lk.forward(ncells, pts, props[i], n0, n1)
        lk.commit(np.ones(nch, np.int32))
        ms.append((time.perf_counter() - t0) * 1e3)
    cl = clocks.stop()
    cpu = acc = None
    if not args.no_cpu:
        try:
            cpu, kept = tt2d_cpu_baseline(grid, settings, data, ncells, pts, props[0], args)
            acc = tt2d_accuracy(lk, data, ncells, pts, props[0], n0, n1, kept)
        except Exception as e:   # the throughput line stands without it
            acc = {"error": "%s: %s" % (type(e).__name__, e)}
    lk.close()
    value = nch * args.steps / (sum(ms) / 1e3)
    # the plain drop-in: one chain per call
    one = TravelTime2DLikelihood(grid, settings, data, nslots=1, ncell_max=100)
    for i in range(3):
        one.forward(ncells[:1], pts[:1], props[i][:1], n0[:1], n1[:1])
    pms = []
    for i in range(max(args.steps, 20)):
        t0 = time.perf_counter()
        one.forward(ncells[i % nch:i % nch + 1], pts[i % nch:i % nch + 1], props[i % len(props)][i % nch:i % nch + 1],
                    n0[:1], n1[:1])
        one.commit(np.ones(1, np.int32))
        pms.append((time.perf_counter() - t0) * 1e3)
    one.close()
    line = {"metric": "2D travel-time forward evals/s, 1 GB300, ttime identical to the reference (fm2d FP64)",
            "value": round(value, 3), "unit": "proposal evals/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(sum(ms) / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 (fm2d in the reference's order)",
            "data": "synthetic (seeded, shapes of the configuration)",
            "config": dict(TT2D_CONFIG, chains=nch),
            "e2e": {"value": round(value, 3), "unit": "proposal evals/s",
                    "h2d_bytes_per_step": int(nch * 100 * 5 * 8 + nch * 4 + nch * 4 * 8),
                    "d2h_bytes_per_step": int(nch * 4 * 8)},
            "note": "host API only (value = e2e): the 2D context has no device-pointer forward",
            "batched_latency_ms": {"p50": round(float(np.percentile(ms, 50)), 3),
                                   "p99": round(float(np.percentile(ms, 99)), 3)},
            "plain": {"value": round(1e3 / float(np.mean(pms)), 3), "unit": "proposal evals/s",
                      "p50_ms": round(float(np.percentile(pms, 50)), 3),
                      "p99_ms": round(float(np.percentile(pms, 99)), 3)},
            "clocks": cl, "valid_models": int((out[:, 3] == 0).sum())}
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if acc is not None:
        line["accuracy"] = acc
    print(json.dumps(line), flush=True)


def tt2d_cpu_baseline(grid, settings, data, ncells, pts, par, args):
    """The oracle's restatement of the 2D path (kd-tree gridding, modrays,
    the likelihood_dd.F90 reductions) for a sample of proposals, one
    proposal per host core at a time (the reference's modrays loop over
    sources is serial)."""
    import concurrent.futures as cf
    import oracle
    orc = oracle.load()
    P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    nx, ny = grid["nx"], grid["ny"]
    src, rev = np.asarray(data["src"]), np.asarray(data["rev"])
    nsrc, nrev = len(src), len(rev)
    rays = np.ascontiguousarray(np.asarray(data["raystat"], np.int32).reshape(nsrc, nrev))
    sx, sy = np.ascontiguousarray(src[:, 0]), np.ascontiguousarray(src[:, 1])
    threads = os.cpu_count() or 1
    nsample = min(len(ncells), 4 * threads)

    def one(c, keep=None):
        n = int(ncells[c])
        sid = np.zeros((nx, ny), np.int32); vp = np.zeros((nx, ny)); vs = np.zeros((nx, ny)); rho = np.zeros((nx, ny))
        orc.orc_kdtree_to_grid(2, n, P(np.ascontiguousarray(pts[c, :n])), P(np.ascontiguousarray(par[c, :n])), nx, ny,
                               1, grid["xmin"], grid["ymin"], 0.0, grid["dx"], grid["dy"], 0.0, 1, nx, 1, ny, 1, 1,
                               P(sid), P(vp), P(vs), P(rho))
        velv = np.ascontiguousarray(np.pad(vp, 1, mode="edge"))
        et = np.zeros((nsrc, nrev))
        orc.orc_modrays(nsrc, P(sx), P(sy), nrev, P(sx), P(sy), P(rays), nx, ny, grid["xmin"], grid["ymin"],
                        grid["dx"], grid["dy"], P(velv), 1, 1, 1, 5, 10, 1, 0.5, P(et), None)
        out = np.zeros(3)
        orc.orc_tt2d_misfit(nsrc, nrev, P(et), P(np.ascontiguousarray(data["ttime"])),
                            P(np.ascontiguousarray(data["sigma"])), P(rays), 0, 0, P(np.zeros(nrev)),
                            P(np.zeros(nrev)), 0, P(np.zeros(2)), P(np.full(2, 0.05)), data["nrays"], P(out))
        if keep is not None:
            keep[c] = (et, out.copy())
        return out[0]

    kept = {}
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda c: one(c, kept), range(nsample)))
    dt = time.perf_counter() - t0
    return {"value": round(nsample / dt, 3), "unit": "proposal evals/s", "cores": threads, "kind": "port",
            "sample": "%d proposals: kd-tree gridding + modrays (16 sources) + misfit, C++ restatement "
                      "of the reference path, one proposal per core" % nsample}, kept


def tt2d_accuracy(lk, data, ncells, pts, par, n0, n1, kept):
    """The GPU context's times and -log L on the oracle's proposals (one
    more forward of that step): every path with data, all sampled chains."""
    rays = np.asarray(data["raystat"], np.int32).reshape(len(data["src"]), len(data["rev"])) == 1
    out = lk.forward(ncells, pts, par, n0, n1)
    errs, err_l = [], 0.0
    for c, (et, eout) in sorted(kept.items()):
        e = np.abs(lk.phase_time(c) - et)[rays]
        errs.append(e)
        err_l = max(err_l, float(abs(out[c, 0] - eout[0]) / abs(eout[0])))
    e = np.concatenate(errs)
    return {"proposals_checked": len(kept), "paths_checked": int(e.size), "max_ttime_err_s": float(e.max()),
            "p99_ttime_err_s": float(np.quantile(e, 0.99)), "frac_paths_within_1e-4_s": float(np.mean(e <= 1e-4)),
            "max_like_rel_err": err_l, "reference": "oracle restatement of the reference path (modrays), FP64"}


SERVED_CONFIG = {
    "workload": "served joint inversion loop: Poisson stream of chains (mean 40 chains/s), kinds drawn uniformly "
                "from 2D travel time (51x51 over 10x10 km, 16 stations, fm2d), surface waves (41x41x31 over "
                "40x40x6 km, 50 stations, 20 periods), body waves (101x101x51 over 50x50x25 km, 200 events, "
                "60 stations, P and S, first-order tiles) and joint surface + body (one 3D model on both), "
                "1,000 proposals per chain, device-resident state, slots sized within a 150 GB budget, "
                "chains evicted on completion",
    "rate_chains_per_s": 40.0, "proposals_per_chain": 1000, "hbm_budget_gb": 150}
SERVED_SLOTS = {"tt2d": 256, "surface": 64, "body": 32, "joint": 32}
# SM shares of the 2D travel-time launches per kind in the batched mode: the
# fm2d grids are persistent, so without a share each launch holds every SM
# until its last block, and the body kinds' 3D passes wait behind it
SERVED_SM_SHARE = "tt2d=0.05,surface=0.15,joint=0.2"


def served_backends(single, slots, priority="none", share=None):
    """The four kinds' backends at the configurations' shapes (single: one
    chain per call on one-slot contexts). priority names the contexts whose
    streams get the device's highest priority in the batched mode: "none",
    "body" (the body kind's context and the joint kind's body context) or
    "body+joint" (the body kind and both of the joint kind's contexts);
    share maps "tt2d", "surface" and "joint" to the SM share of that kind's
    2D travel-time launches (the joint kind's surface context) in the
    batched mode. Returns (backends, bytes per kind)."""
    import torch
    from mctomo_gb300 import BodyLikelihood, SurfaceLikelihood, TravelTime2DLikelihood, serving, synthetic
    rng = np.random.default_rng(SEED + 6)
    used = {}

    def sized(kind, make):
        torch.cuda.synchronize()
        f0 = torch.cuda.mem_get_info()[0]
        obj = make()
        torch.cuda.synchronize()
        used[kind] = used.get(kind, 0) + max(0, f0 - torch.cuda.mem_get_info()[0])
        return obj
    n = {k: (1 if single else v) for k, v in slots.items()}
    g2, s2, d2 = synthetic.tt2d_workload(rng)
    nm, pr = synthetic.serving_models("tt2d", g2, 100, (4, 100))
    tt2d = serving.TT2DBackend(sized("tt2d", lambda: TravelTime2DLikelihood(g2, s2, d2, n["tt2d"], 100)), n["tt2d"],
                               nm, pr, single=single)
    gs, ss, ds = synthetic.surface_workload(rng)
    ss["tt_precision"] = 0            # FP64 fm2d: times identical to the reference
    nm, pr = synthetic.serving_models("surface", gs, 400, (10, 400))
    surf = serving.SurfaceBackend(sized("surface", lambda: SurfaceLikelihood(gs, ss, ds, n["surface"], 400)),
                                  n["surface"], nm, pr, len(ds["freqs"]), single=single)
    gb, sb, db, ev = synthetic.body_workload(rng)
    sb["order"] = 0
    sb["solver"] = 0x10
    nm, pr = synthetic.serving_models("body", gb, 800, (20, 800))
    body = serving.BodyBackend(sized("body", lambda: BodyLikelihood(gb, sb, db, n["body"], 800)), n["body"], nm, pr,
                               ev, single=single)
    nmj, prj = synthetic.serving_models("joint", gb, 800, (20, 800))
    js = serving.SurfaceBackend(sized("joint", lambda: SurfaceLikelihood(gs, ss, ds, n["joint"], 800)), n["joint"],
                                nmj, prj, len(ds["freqs"]), single=single)
    jb = serving.BodyBackend(sized("joint", lambda: BodyLikelihood(gb, sb, db, n["joint"], 800)), n["joint"], nmj,
                             prj, ev, single=single)
    joint = serving.JointBackend(js, jb)
    if not single and share:
        # 2D travel-time kernels hold their SMs for the whole launch; a share
        # per kind leaves SMs free for the body kinds' short 3D passes
        for kind, obj in (("tt2d", tt2d), ("surface", surf), ("joint", js)):
            if kind in share:
                obj.set_sm_share(share[kind])
    if not single and priority != "none":
        # The body kinds wait on the host between the 3D solver's passes; a
        # high-priority stream keeps their short launches from queueing
        # behind the 2D and surface kinds' long travel-time kernels.
        body.set_priority(True)
        if priority == "body":
            jb.set_priority(True)
        else:
            joint.set_priority(True)
    return {"tt2d": tt2d, "surface": surf, "body": body, "joint": joint}, used


def served_trace_check(traces):
    """Every chain that ran in both legs has the same seed, so its -log L
    trace (one value per step: the state after the Metropolis decision) is
    the same served and plain as long as each evaluation is: the exact kinds
    (FP64 fm2d) must agree bit for bit; the body kinds' tile solver may move
    a time by a few fixed-point units with the other chains of a call, which
    can flip a later decision. Per kind: the steps compared (up to the first
    step differing by more than 1e-6 relative, where the traces part), the
    share identical, the largest relative difference before they part, and
    the chains whose traces parted."""
    out = {}
    for cid, (kind, a) in traces["served"].items():
        if cid not in traces["plain"]:
            continue
        b = traces["plain"][cid][1]
        o = out.setdefault(kind, {"chains_compared": 0, "steps_compared": 0, "identical_steps": 0,
                                  "max_rel_diff": 0.0, "chains_parted": 0})
        o["chains_compared"] += 1
        for x, y in zip(a, b):
            d = abs(x - y) / max(abs(y), 1e-300)
            if d > 1e-6:
                o["chains_parted"] += 1
                break
            o["steps_compared"] += 1
            o["identical_steps"] += int(x == y)
            o["max_rel_diff"] = max(o["max_rel_diff"], d)
    for o in out.values():
        o["identical_frac"] = round(o["identical_steps"] / max(o["steps_compared"], 1), 6)
    return out


def parse_share(spec):
    """'kind=share,...' (kinds tt2d, surface, joint) -> dict; 'none' -> {}."""
    if not spec or spec == "none":
        return {}
    out = {}
    for item in spec.split(","):
        k, v = item.split("=")
        if k not in ("tt2d", "surface", "joint"):
            raise SystemExit("--served-sm-share: unknown kind %r" % k)
        out[k] = float(v)
    return out


def run_served(args):
    """Configuration 5: the served loop (continuous batching over the four
    kinds' contexts, one worker thread and stream per kind) on a Poisson
    stream, then the same stream through the plain drop-in (one-slot
    contexts, one call per proposal). Per-proposal latency is the time from
    a proposal's submission to its result."""
    import torch
    from mctomo_gb300 import serving
    names = ["tt2d", "surface", "body", "joint"]
    rng = np.random.default_rng(SEED + 7)
    dur, warm = args.served_seconds, args.served_seconds / 3.0
    arrivals = serving.poisson_arrivals(rng, SERVED_CONFIG["rate_chains_per_s"], dur, names)
    res, traces = {}, {}
    share = parse_share(args.served_sm_share)
    slots = dict(SERVED_SLOTS)
    for item in filter(None, args.served_slots.split(",")):
        k, v = item.split("=")
        if k not in slots:
            raise SystemExit("--served-slots: unknown kind %r" % k)
        slots[k] = int(v)
    for plain in (False, True) if not args.served_only else (False,):
        backends, used = served_backends(plain, slots, args.served_priority, share)
        if sum(used.values()) > SERVED_CONFIG["hbm_budget_gb"] * 1e9:
            raise SystemExit("served contexts exceed the HBM budget: %s" % used)
        # one warm-up step per kind outside the stream
        for k in names:
            b = backends[k]
            mdl = [b.new_model(np.random.default_rng(1))]
            b.forward([0], mdl)
            b.commit([0], [0])
        torch.cuda.synchronize()
        workers = [serving.Worker(k, backends[k], SERVED_CONFIG["proposals_per_chain"], plain=plain) for k in names]
        clocks = Clocks(0)
        clocks.start()
        stats, chains = serving.run_stream(workers, arrivals, dur, (warm, dur), seed=SEED)
        stats["clocks"] = clocks.stop()
        stats["device_bytes"] = {k: int(v) for k, v in used.items()}
        res["plain" if plain else "served"] = stats
        traces["plain" if plain else "served"] = {ch.cid: (ch.kind, list(ch.trace)) for ch in chains if ch.trace}
        del backends, workers
        torch.cuda.synchronize()
    sv = res["served"]
    pl = res.get("plain", {"evals_per_s": 0.0, "kinds": {}})
    line = {"metric": "served proposal evals/s & p99 proposal latency, mixed stream, 1 GB300",
            "value": round(sv["evals_per_s"], 3), "unit": "proposal evals/s", "n_gpus": 1, "steps": None,
            "warmup": None, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64 dispersion polish, f32 bracketing; f64 fm2d (reference order); int32 fixed-point 3D tiles",
            "data": "synthetic (seeded, shapes of configurations 1-3)",
            "config": dict(SERVED_CONFIG, slots=slots, seconds=dur, measured_window_s=[round(warm, 1), dur],
                           arrivals=len(arrivals), high_priority_streams=args.served_priority,
                           sm_share=share or "whole device"),
            "served": sv, "plain": pl,
            "served_over_plain": round(sv["evals_per_s"] / pl["evals_per_s"], 3) if pl["evals_per_s"] else None,
            "accuracy": served_trace_check(traces) if "plain" in traces else None,
            "clocks": sv["clocks"]}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Small fixed cases of the hot kernels, for profilers (--case). Each prints one
# line and exits 0.
#   fm2d: M Voronoi phase maps of 41 x 41 vertices (1 km spacing), 50 stations
#     between 2 and 38 km, every station pair once, source refinement 4 x over
#     8 cells (the surface likelihood's fm2d settings); R calls of
#     mct_modrays_batch.
#   eik3: 8 velocity grids of 101 x 101 x 51 nodes (0.5 km), 120 solves.
#   eik3heap: the exact heap march, N solves (default 8) on 4 Voronoi grids of
#     51 x 51 x 26 nodes (0.5 km, velocities 3-7.5 km/s).
#   disp: N layered columns (12-40 layers, no low-velocity layers), 20 Rayleigh
#     fundamental-mode phase periods log-spaced 0.5-5 s, search increment 1e-3
#     km/s; with --case-study, N columns of the dispersion-precision study
#     (10 % low-velocity-layer chance, 60 periods 0.2-20 s, fundamental and
#     first overtone, phase and group).
#   grid: nearest-nucleus gridding of a 101 x 101 x 51 grid over 50 x 50 x 25
#     km from 800 nuclei.
#   tiles: the body-wave forward (101 x 101 x 51 grid, 200 events, 60
#     stations, P and S, first order) of N chains with each configuration of
#     the 3D tile solver forced in turn, then the tuned one.
# ---------------------------------------------------------------------------
def _case_modules():
    from mctomo_gb300 import forward, synthetic
    return forward, synthetic


def case_fm2d(precision=1, maps=16, repeat=2):
    forward, synthetic = _case_modules()
    rng = np.random.default_rng(0)
    nvx = nvz = 41
    st = rng.uniform(2.0, 38.0, (50, 2))
    srs = np.triu(np.ones((50, 50), np.int32), 1)
    velv = synthetic.voronoi_phase_maps(rng, maps, nvx, nvz, 1.0, 1.0)
    for _ in range(repeat):
        t0 = time.perf_counter()
        tt = forward.modrays_batch(st, st, srs, nvx, nvz, 0.0, 0.0, 1.0, 1.0, velv, sgdl=4, sgs=8,
                                   precision=precision)
        dt = time.perf_counter() - t0
    print(f"fm2d precision={precision} maps={maps} solves={maps * 49} last_call_s={dt:.4f} t01={tt[0, 0, 1]:.6f}")


def case_eik3(order=0):
    forward, synthetic = _case_modules()
    rng = np.random.default_rng(1)
    nx, ny, nz = 101, 101, 51
    h = (0.5, 0.5, 0.5)
    lo = (0.0, 0.0, 0.0)
    z = np.arange(nz) * h[2]
    vels = np.stack([np.broadcast_to(3.0 + 0.08 * z * (1 + 0.1 * g), (nx, ny, nz)).copy() *
                     (1 + 0.05 * rng.standard_normal((nx, ny, nz))) for g in range(8)])
    nsolve = 120
    grid = (np.arange(nsolve) % 8).astype(np.int32)
    srcs = rng.uniform([2, 2, 1], [48, 48, 20], (nsolve, 3))
    rev = rng.uniform([2, 2, 0], [48, 48, 0.5], (60, 3))
    t0 = time.perf_counter()
    tt, _, passes = forward.eikonal3d_batch(vels, h, lo, grid, srcs, rev, order=order)
    dt = time.perf_counter() - t0
    print(f"eik3 order={order} solves={nsolve} passes={passes} call_s={dt:.4f} t00={tt[0, 0]:.6f}")


def case_eik3heap(order=1, solves=8):
    forward, synthetic = _case_modules()
    rng = np.random.default_rng(4)
    shape = (51, 51, 26)
    h = (0.5, 0.5, 0.5)
    lo = np.zeros(3); hi = (np.array(shape) - 1) * 0.5
    X, Y, Z = np.meshgrid(*[np.arange(k) * 0.5 for k in shape], indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    vels = []
    for g in range(4):
        pts, par = synthetic.voronoi_model_3d(rng, 120, lo, hi, (3.0 / 1.73, 7.5 / 1.73))
        d = ((nodes[:, None, :] - pts[None]) ** 2).sum(-1)
        vels.append((par[:, 1] * 1.73)[d.argmin(1)].reshape(shape))
    vels = np.stack(vels)
    grid = (np.arange(solves) % 4).astype(np.int32)
    srcs = rng.uniform([1, 1, 0], [24, 24, 0.2], (solves, 3))
    rev = rng.uniform([1, 1, 1], [24, 24, 12], (40, 3))
    t0 = time.perf_counter()
    tt, _, _ = forward.eikonal3d_batch(vels, h, lo, grid, srcs, rev, order=order, solver="heap")
    dt = time.perf_counter() - t0
    print(f"eik3heap order={order} solves={solves} call_s={dt:.4f} t00={tt[0, 0]:.6f}")


def case_disp(precision=1, columns=4096, study=False):
    forward, synthetic = _case_modules()
    rng = np.random.default_rng(2)
    if study:
        nl, thk, vp, vs, rho = synthetic.layered_columns(rng, columns, nl_range=(12, 40), lvl_prob=0.1)
        periods = np.geomspace(0.2, 20.0, 60)
        kw = dict(mode=2, multimode=True)
    else:
        nl, thk, vp, vs, rho = synthetic.layered_columns(rng, columns, lvl_prob=0.0)
        periods = np.geomspace(0.5, 5.0, 20)
        kw = {}
    t0 = time.perf_counter()
    cp, _, ierr, cnt = forward.surfdisp_batch(nl, thk, vp, vs, rho, periods, 2, int(study), 1e-3,
                                              precision=precision, **kw)
    dt = time.perf_counter() - t0
    print(f"disp precision={precision} columns={columns} study={int(study)} call_s={dt:.4f} ierr={int((ierr != 0).sum())} "
          f"evals_fp64={cnt[0]} evals_fp32={cnt[1]} cp00={cp[0, 0, 0]:.6f}")


def case_grt(modetype=1, columns=20, periods=4):
    """A small generalized R/T case for ncu: the first columns of a seeded
    draw that route to the generalized R/T search, a few periods."""
    forward, synthetic = _case_modules()
    rng = np.random.default_rng(11)
    nl, thk, vp, vs, rho = synthetic.layered_columns(rng, 64 * columns, nl_range=(12, 40), lvl_prob=0.1)
    thk, vp, vs, rho = (np.ascontiguousarray(x, np.float64) for x in (thk, vp, vs, rho))
    sel = np.where(forward.surfmodes_route(nl, vp, vs, modetype) == 1)[0][:columns]
    freqs = 1.0 / np.geomspace(0.2, 20.0, 60)[::max(1, 60 // periods)][:periods]
    t0 = time.perf_counter()
    ph, gr, ierr, nev = forward.grt_batch(nl[sel], thk[sel], vp[sel], vs[sel], rho[sel], freqs,
                                          forward.modes_para(modetype, 1))
    dt = time.perf_counter() - t0
    print(f"grt modetype={modetype} columns={len(sel)} periods={len(freqs)} call_s={dt:.4f} evals={nev} "
          f"ierr={int((ierr != 0).sum())} ph00={ph[0, 0]:.6f}")


def case_grid():
    forward, synthetic = _case_modules()
    rng = np.random.default_rng(3)
    lo = np.zeros(3); hi = np.array([50.0, 50.0, 25.0])
    shape = (101, 101, 51)
    st = (hi - lo) / (np.array(shape) - 1)
    pts, par = synthetic.voronoi_model_3d(rng, 800, lo, hi, (1.7, 4.3))
    t0 = time.perf_counter()
    sid, _, _, _ = forward.kdtree_to_grid(pts, par, *shape, lo, st)
    dt = time.perf_counter() - t0
    print(f"grid nodes={sid.size} nuclei=800 call_s={dt:.4f} sid0={int(sid.ravel()[0])}")


def case_tiles(chains=32):
    forward, synthetic = _case_modules()
    from mctomo_gb300 import BodyLikelihood, lib
    L = lib()
    rng = np.random.default_rng(5)
    grid, settings, data, ev = synthetic.body_workload(rng)
    settings["order"] = 0
    settings["solver"] = 0x10
    lo = np.zeros(3); hi = np.array([50.0, 50.0, 25.0]); ncell_max = 800
    ncells = rng.integers(20, ncell_max + 1, chains).astype(np.int32)
    pts = np.zeros((chains, ncell_max, 3)); par = np.zeros((chains, ncell_max, 3))
    for c in range(chains):
        p, q = synthetic.voronoi_model_3d(rng, int(ncells[c]), lo, hi, (3.0 / 1.73, 7.5 / 1.73))
        q[:, 0] = q[:, 1] * 1.73
        pts[c, :ncells[c]] = p; par[c, :ncells[c]] = q
    locs = np.repeat(ev[None], chains, 0)
    n0 = np.zeros((chains, 2)); n1 = np.full((chains, 2), 0.05)
    lk = BodyLikelihood(grid, settings, data, nslots=chains, ncell_max=ncell_max)
    old = L.mct_eik3_tile_config(-1, 0, 0, 0, 0)
    ref = None
    for cfg in list(range(48)) + [-1]:
        L.mct_eik3_tile_config(cfg, 0, 0, 0, 0)
        lk.forward(ncells, pts, par, locs, n0, n1)
        t0 = time.perf_counter()
        out = lk.forward(ncells, pts, par, locs, n0, n1)
        dt = time.perf_counter() - t0
        ref = out if ref is None else ref
        print(f"tiles cfg={cfg} chains={chains} forward_s={dt:.3f} passes={lk.phase_time(0)[1]} "
              f"max_like_diff={float(np.max(np.abs(out[:, 0] - ref[:, 0]))):.3g}", flush=True)
    print(f"tiles tuned_cfg={L.mct_eik3_tile_config(-2, 101, 101, 51, 0)}")
    L.mct_eik3_tile_config(old, 0, 0, 0, 0)
    lk.close()


def run_case(a):
    if a.case == "fm2d":
        case_fm2d(a.case_precision, a.case_maps, a.case_repeat)
    elif a.case == "eik3":
        case_eik3(a.case_order or 0)
    elif a.case == "eik3heap":
        case_eik3heap(1 if a.case_order is None else a.case_order, a.case_solves)
    elif a.case == "disp":
        case_disp(a.case_precision, a.case_columns, a.case_study)
    elif a.case == "tiles":
        case_tiles(a.chains)
    elif a.case == "grt":
        case_grt(1 if a.case_order is None else a.case_order, min(a.case_columns, 128))
    else:
        case_grid()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--tt-precision", type=int, default=0,
                    help="surface workload: fm2d arithmetic (0 FP64 exact, 1 double-float, 2 fixed point)")
    ap.add_argument("--no-variant", action="store_true", help="surface workload: skip the double-float variant")
    ap.add_argument("--workload", default="surface",
                    choices=["surface", "body", "disp", "tt2d", "served", "dropin", "grt"])
    ap.add_argument("--served-seconds", type=float, default=60.0, help="served workload: stream length (s)")
    ap.add_argument("--served-priority", default="none", choices=["none", "body", "body+joint"],
                    help="served workload: contexts whose streams run at the device's highest priority")
    ap.add_argument("--served-sm-share", default=SERVED_SM_SHARE,
                    help="served workload: SM share of the 2D travel-time launches per kind, "
                         "e.g. tt2d=0.15,surface=0.25,joint=0.2 (none: whole device)")
    ap.add_argument("--served-only", action="store_true", help="served workload: skip the plain leg")
    ap.add_argument("--served-slots", default="", help="served workload: slots per kind, e.g. body=48,joint=32")
    ap.add_argument("--chains2d", type=int, default=256, help="tt2d workload: chains per step")
    ap.add_argument("--columns", type=int, default=262144, help="disp workload: columns")
    ap.add_argument("--disp-sample", type=int, default=512, help="disp workload: columns checked by the oracle")
    ap.add_argument("--love-cols", type=int, default=0, help="disp workload: columns with Love waves (0: all)")
    ap.add_argument("--grt-cols", type=int, default=262144, help="grt workload: columns drawn (about 10%% routed)")
    ap.add_argument("--grt-sample", type=int, default=128, help="grt workload: routed columns per wave the oracle checks")
    ap.add_argument("--chains", type=int, default=32, help="body workload: chains per step")
    ap.add_argument("--order", type=int, default=0, help="body workload: eikonal order")
    ap.add_argument("--body-sample", type=int, default=2, help="body workload: proposals checked by the oracle")
    ap.add_argument("--dropin-threads", type=int, default=16, help="dropin workload: host threads")
    ap.add_argument("--dynamic", action="store_true",
                    help="body workload: keep the stations' travel-time fields and time location steps on them")
    ap.add_argument("--solver", default=None, choices=["tiles", "heap"],
                    help="body workload: 3D solver (default: heap march for order 1, tiles for order 0)")
    ap.add_argument("--case", default=None, choices=["fm2d", "eik3", "eik3heap", "disp", "grid", "tiles", "grt"],
                    help="run one small fixed case of a hot kernel (for profilers) instead of a workload")
    ap.add_argument("--case-precision", type=int, default=1)
    ap.add_argument("--case-maps", type=int, default=16)
    ap.add_argument("--case-repeat", type=int, default=2)
    ap.add_argument("--case-solves", type=int, default=8)
    ap.add_argument("--case-columns", type=int, default=4096)
    ap.add_argument("--case-order", type=int, default=None)
    ap.add_argument("--case-study", action="store_true")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    if args.workload in ("body", "disp", "tt2d", "served", "dropin", "grt"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the surface workload"}))
        elif args.workload == "served":
            run_served(args)
        elif args.workload == "dropin":
            run_dropin(args)
        elif args.workload == "body":
            run_body(args)
        elif args.workload == "disp":
            run_disp(args)
        elif args.workload == "grt":
            run_grt(args)
        else:
            run_tt2d(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

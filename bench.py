"""Benchmark of the GRMHD fluid hot path on one GB300 (per rank).

Workload: the 256^3 single-meshblock shear layer (Minkowski, ideal gas
Gamma = 5/3, WENO5-Z + HLL, MHD, periodic), seeded synthetic state.  One
bench step = one full Heun RK2 timestep of the reference's stage sequence
(two stages: sources, fluxes, FluxCT, divergence + update, con2prim over the
whole block, ghost exchange, con2prim again; then the face-speed timestep
estimate).  The metric is zone-updates/s: interior zones advanced one full
RK2 timestep per second.

  value      device-resident state, CUDA events around K steps
  e2e        the same steps through the C ABI with the state in pinned host
             memory: every step copies prims + cons to the device, runs, and
             copies prims + cons back, all inside the timed region (copies on
             two copy streams overlap the previous/next step's compute)
  roofline   CalculateFluxes (the dominant kernels): algorithmic bytes per
             launch / measured launch time vs the measured HBM copy peak; an
             FP64 section relates the same launches to the measured FP64 peak
  cpu_baseline  the oracle (CPU restatement of the reference path, its -O3
             timing build) timed on a 128^3 sample of the same state with all
             host threads

  batched    1024 uneven periodic blocks (edges 16/32/64, MP5 + HLL): RK2
             steps through phx_stage_batched (persistent work-list launches
             replayed as CUDA graphs) against the same steps block by block
  torus      magnetised torus on a 384^3 FMKS mesh of uneven blocks: the plain
             GPU step (block-by-block launches, reference con2prim start)
             against the learned start + batched graphs
  c2p        con2prim over 5e7 independent FMKS Kerr-Schild zones at tolerance
             1e-10: zones/s and root-find iterations with the reference's
             start (plain) and with the learned start (network trained on
             the GPU on 1e7 separately seeded pairs, 20 epochs, before timing)

The sections' full results are printed as one {"detail": ...} line before the
result line, which carries their headline numbers under "sections".

--impl reference runs the reference's CPU path (the oracle port, its timing
build) on all host cores: each step is one RK2 timestep of the same 256^3
block.
Multi-GPU: independent replicas (one block per rank, weak scaling); the only
cross-rank operations are the timing barriers.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GRMHD zone-updates/s on 1 GB300; con2prim zones/s learned-guess vs plain @1e-10"
UNIT = "zone-updates/s"
LAUNCHES_DT = 3


def c2p_launches(nzones: int, learned: bool = False) -> int:
    """Kernel launches of one con2prim call: per chunk of C2P_CHUNK zones a
    root-find launch and a retry launch (plus the bracket launch when
    learned)."""
    from phoebus_gb300 import abi

    chunks = -(-nzones // abi.C2P_CHUNK)
    return chunks * (3 if learned else 2)


def stage_launches(n: int, ng: int = 4) -> int:
    """Kernel launches of one RK stage on an n^3 periodic MHD block without
    floors or fixups: sources 1, fluxes 3, FluxCT 2, update 1, ghosts 1, and
    two con2prim calls over the entire block."""
    return 8 + 2 * c2p_launches((n + 2 * ng) ** 3)


def parse():
    a = argparse.ArgumentParser()
    a.add_argument("--gpus", type=int, default=1)
    a.add_argument("--steps", type=int, default=5)
    a.add_argument("--warmup", type=int, default=3)
    a.add_argument("--impl", default="ours", choices=["ours", "reference"])
    a.add_argument("--n", type=int, default=256)
    a.add_argument("--cpu-n", type=int, default=128,
                   help="edge of the block the cpu_baseline leg of this arm times (a sample of the workload)")
    a.add_argument("--ref-n", type=int, default=0,
                   help="--impl reference: block edge (0 = the workload's own --n)")
    a.add_argument("--exact", action="store_true", help="time the parity (no-FMA) build")
    a.add_argument("--no-e2e", action="store_true")
    a.add_argument("--no-cpu", action="store_true")
    a.add_argument("--no-c2p", action="store_true", help="skip the con2prim learned-vs-plain section")
    a.add_argument("--c2p-zones", type=float, default=5e7)
    a.add_argument("--train-pairs", type=float, default=1e7)
    a.add_argument("--train-epochs", type=int, default=20)
    a.add_argument("--no-batched", action="store_true", help="skip the uneven-meshblock section")
    a.add_argument("--batched-blocks", type=int, default=1024)
    a.add_argument("--no-torus", action="store_true", help="skip the torus section")
    a.add_argument("--torus-n", type=int, default=384)
    a.add_argument("--torus-steps", type=int, default=2)
    a.add_argument("--section-steps", type=int, default=3, help="RK2 steps per timed round (batched section)")
    a.add_argument("--section-rounds", type=int, default=2,
                   help="interleaved timed rounds per arm (batched and torus sections)")
    a.add_argument("--no-m1", action="store_true", help="skip the radiation M1 section")
    a.add_argument("--m1-only", action="store_true",
                   help="run only the radiation M1 section and print its JSON (profiling)")
    a.add_argument("--m1-n", type=int, default=128)
    a.add_argument("--m1-steps", type=int, default=3)
    a.add_argument("--m1-cpu-n", type=int, default=64)
    return a.parse_args()


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if args.impl == "ours" else "gloo"
        if args.impl == "ours":
            import torch

            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(ws, v, device=None):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        import statistics

        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def flux_bytes(n, ng=4, exact=False):
    """Algorithmic HBM bytes of one CalculateFluxes call (three launches) on
    an n^3 block: each direction reads the reconstructed primitives of every
    cell its stencils touch (9 in the production build, which takes gamma1 as
    the ideal gas's constant Gamma; the exact build reads all 10) and writes
    8 fluxes + 1 signal speed per face it computes."""
    n1t = n + 2 * ng
    t = n + 2  # transverse face range [s-1, e+1]
    cells = n1t * t * t  # stencil cells per direction (full pencil, +-1 layer)
    faces = (n + 1) * t * t
    nrec = 10 if exact else 9
    return 3 * (nrec * cells + 9 * faces) * 8


def bench_c2p(ctx, args, dev):
    """Independent-zone con2prim at tolerance 1e-10 on seeded FMKS Kerr-Schild
    zones (spin 0.9375): zones/s and FP64 root-find iterations per zone with
    the reference's start (plain) and with the learned start, the network
    trained first on the GPU on separately seeded pairs.  Each timed run
    starts from c2p_mu = 0 (the plain start's guess) and the pristine
    conserved state; the state (about 18 GB for 5e7 zones) is far larger
    than L2."""
    import torch

    from phoebus_gb300 import abi, learned, states

    N = int(args.c2p_zones)
    p = abi.default_params(gm1=1.0 / 3.0)
    p.c2p_tol, p.c2p_max_iter = 1e-10, 100
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    opts = abi.default_train_opts(epochs=args.train_epochs)
    losses = learned.train(ctx, p, n=int(args.train_pairs), opts=opts, device=dev)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    prim = torch.empty((abi.NPRIM, N), dtype=torch.float64, device=dev)
    cons = torch.empty((abi.NCONS, N), dtype=torch.float64, device=dev)
    geom = torch.empty((abi.GEOM_NLOC, N), dtype=torch.float64, device=dev)
    chunk = 10_000_000
    for s0 in range(0, N, chunk):
        m = min(chunk, N - s0)
        pr, co, ge = learned.kerr_zone_set(ctx, p, m, states.SEED + 4, dev, start=s0)
        prim[:, s0:s0 + m] = pr
        cons[:, s0:s0 + m] = co
        geom[:, s0:s0 + m] = ge
        del pr, co, ge
    cons0 = cons.clone()
    fail = torch.empty(N, dtype=torch.float64, device=dev)
    sig = torch.empty((3, N), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    out = {}
    for name, lrn in (("plain", False), ("learned", True)):
        times = []
        for rep in range(4):  # one untimed warm-up, three timed
            prim[abi.PMU].zero_()
            cons.copy_(cons0)
            ctx.c2p_stats(reset=True)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.ConservedToPrimitiveZones(p, cons, prim, geom, fail=fail, cell_sig=sig, learned=lrn)
            e1.record(stream)
            torch.cuda.synchronize()
            if rep:
                times.append(e0.elapsed_time(e1))
            st = ctx.c2p_stats(reset=True)
        ctx.check()
        ms = sorted(times)[len(times) // 2]
        out[name] = {"zones_per_s": N / (ms * 1e-3), "ms": ms, "iterations_per_zone": st["iterations"] / N,
                     "residual_evals_per_zone": st["residual_evals"] / N, "failures": st["failures"],
                     "unbracketed": st["unbracketed"], "gpu_launches": c2p_launches(N, lrn)}
        if lrn:
            out[name]["learned_accepted_frac"] = st["learned_accepted"] / N
    del prim, cons, geom, cons0, fail, sig
    torch.cuda.empty_cache()
    out["learned_over_plain"] = out["learned"]["zones_per_s"] / out["plain"]["zones_per_s"]
    out["zones"] = N
    out["tolerance"] = 1e-10
    out["workload"] = ("independent zones, FMKS Kerr-Schild a=0.9375 (no pole derefinement), r in [1.5, 50], "
                       "theta in (0, pi), log10 rho in [-6, 0], log10 u/rho in [-4, 1], W in [1, 10], "
                       "sigma in [1e-4, 1e2], ideal gas Gamma 4/3; cons from the library's prim2con")
    out["training"] = {"pairs": int(args.train_pairs), "epochs": args.train_epochs, "batch": opts.batch,
                       "seconds": t_train, "final_loss": losses[-1], "first_epoch_loss": losses[0],
                       "optimizer": "AdamW, cosine lr 3e-3 -> 0"}
    return out


def batched_params():
    """Uneven-block workload: MP5 + HLL, Gamma 4/3, MHD; ConstantRhoSie
    floors, c2p fixup and ceilings on (the per-zone random state develops
    failed inversions within a few steps without them)."""
    from phoebus_gb300 import abi

    p = abi.default_params(Gamma=4.0 / 3.0, recon="mp5", riemann="hll", c2p_tol=1e-10, c2p_max_iter=100)
    p.enable_floors, p.enable_c2p_fixup, p.enable_ceilings = 1, 1, 1
    p.rho0_floor, p.sie0_floor = 1e-8, 1e-8
    return p


def _timed_rounds(arms, restore, rounds, stream):
    """Run every arm (name, step function, steps per round) from the same
    restored state, interleaved over rounds; per arm the median over rounds
    of the mean ms per step.  Each arm's first call (plan build, autotune,
    graph capture) happens before its timed rounds."""
    import statistics

    import torch

    for _, fn, _ in arms:
        restore()
        fn()
    ms = {name: [] for name, _, _ in arms}
    for _ in range(rounds):
        for name, fn, k in arms:
            restore()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(k):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms[name].append(e0.elapsed_time(e1) / k)
    return {name: statistics.median(v) for name, v in ms.items()}, ms


def bench_batched(ctx, args, dev, learned_ready=False):
    """1024 periodic blocks with edges from {16, 32, 64} (p = 0.5, 0.35,
    0.15), per-zone random primitives; one RK2 step = two batched stages
    (each a captured CUDA graph of persistent work-list launches).  Compared
    with the same steps issued block by block through phx_stage.  Every arm
    starts from the same snapshot of the initialised state; the batched arms
    are interleaved over rounds and reported as the median round."""
    import torch

    from phoebus_gb300 import states
    from phoebus_gb300.block import Block

    p = batched_params()
    blocks = states.uneven_blocks(args.batched_blocks, device=dev)
    for b in blocks:
        ctx.Initialize(p, b)
    ctx.check()
    zones = sum(b.nx[0] * b.nx[1] * b.nx[2] for b in blocks)
    dt = 0.2 * min(ctx.EstimateTimestepBlock(p, b, False).item() for b in blocks)
    seconds = [torch.zeros_like(b["cons"]) for b in blocks]
    # the stage inputs: prims, cons, and the second-stage buffers, whose ghost
    # zones (from the previous step's exchange) the first con2prim of a stage
    # reads, as the reference's does
    snap = [(b["prim"].clone(), b["cons"].clone(), s2.clone()) for b, s2 in zip(blocks, seconds)]

    def restore():
        for b, s2, (pr, co, sc) in zip(blocks, seconds, snap):
            b["prim"].copy_(pr)
            b["cons"].copy_(co)
            s2.copy_(sc)

    bases = [b["cons"] for b in blocks]
    stage2 = []
    for b, s2 in zip(blocks, seconds):
        c = Block(b.nx, b.ng, b.ndim, b.xmin, b.dx, backend="torch", device=dev, arrays=dict(b.arrays))
        c.arrays["cons"] = s2
        stage2.append(c)

    def step_batched(learned=False):
        ctx.StageBatched(p, blocks, bases, seconds, 1.0, dt, learned=learned)
        ctx.StageBatched(p, stage2, bases, bases, 0.5, dt, learned=learned)

    def step_batched_learned():
        step_batched(True)

    def step_blocks():
        for b, b2, s2 in zip(blocks, stage2, seconds):
            ctx.Stage(p, b, b["cons"], s2, 1.0, dt)
            ctx.Stage(p, b2, b["cons"], b["cons"], 0.5, dt)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    step_batched()  # builds both plans: work lists, autotune, graph capture
    torch.cuda.synchronize()
    t_plan = time.perf_counter() - t0
    info = ctx.batch_info()
    stream = torch.cuda.current_stream()
    k = args.section_steps
    arms = [("batched", step_batched, k)]
    if learned_ready:
        arms.append(("batched_learned", step_batched_learned, k))
    med, per_round = _timed_rounds(arms, restore, args.section_rounds, stream)
    res = {}
    for name, _, _ in arms:
        res[name] = {"zone_updates_per_s": zones / (med[name] * 1e-3), "ms_per_step": med[name], "steps": k,
                     "rounds_ms": per_round[name]}
    # statistics of one step of each arm from the snapshot
    for name, fn, _ in arms:
        restore()
        ctx.c2p_stats(reset=True)
        fn()
        st = ctx.c2p_stats(reset=True)
        if st["zones"]:
            res[name]["c2p_iterations_per_zone"] = st["iterations"] / st["zones"]
            res[name]["c2p_learned_accepted_frac"] = st["learned_accepted"] / st["zones"]
    pb, _ = _timed_rounds([("per_block", step_blocks, 1)], restore, 1, stream)
    res["per_block"] = {"zone_updates_per_s": zones / (pb["per_block"] * 1e-3), "ms_per_step": pb["per_block"],
                        "steps": 1}
    ctx.check()
    nan = sum(int(torch.isnan(b["prim"][0]).sum()) for b in blocks)
    del blocks, seconds, bases, stage2, snap
    torch.cuda.empty_cache()
    from collections import Counter

    sizes = Counter(states.uneven_block_sizes(args.batched_blocks))
    out = {"workload": f"{args.batched_blocks} periodic blocks, edges {dict(sorted(sizes.items()))}, Minkowski, "
                       "MP5 + HLL, MHD, Gamma 4/3, per-zone random state, floors + c2p fixup on",
           "interior_zones": zones, **res, "batched_over_per_block":
               res["batched"]["zone_updates_per_s"] / res["per_block"]["zone_updates_per_s"],
           "plan_seconds": t_plan, "tuning": info, "nan_rho_zones": nan,
           "inputs": "every arm from the same snapshot of the initialised state; batched arms interleaved over "
                     f"{args.section_rounds} rounds of {k} steps, median round",
           "graph": "one CUDA graph per stage kind; nodes per graph as in tuning.graph_nodes"}
    if "batched_learned" in res:
        out["learned_over_batched"] = (res["batched_learned"]["zone_updates_per_s"] /
                                       res["batched"]["zone_updates_per_s"])
    return out


def bench_torus(ctx, args, dev, learned_ready=False):
    """Magnetised FM torus (r_in 6, r_max 12, Gamma 13/9, beta 100, 4%
    pressure noise) on an n^3 FMKS Kerr-Schild mesh (a = 0.9375, X1 in
    [ln 1.2, ln 250]) split into uneven blocks (edges 32..96 per axis),
    WENO5-Z + HLL, ExpX1RhoSie floors, MHD floors, ceilings, c2p fixup,
    outflow X1/X2, periodic X3.  RK2 steps: the plain GPU step (every phase
    launched block by block, the reference's con2prim start) against the
    learned start + batched persistent launches replayed as CUDA graphs."""
    import torch

    from phoebus_gb300 import learned, torus

    p = torus.torus_params()
    mesh = torus.torus_mesh(n=args.torus_n)
    geo = torus.torus_geometry()
    blocks = mesh.make_blocks(dev, geo)
    setup_s = []
    for _ in range(2):  # the first fill also loads torch's kernels; the second is the setup cost
        torch.cuda.synchronize()
        t_setup = time.perf_counter()
        info = torus.fill_torus(ctx, p, mesh, blocks)  # tables, FM state, field, p2c, exchange, con2prim on the GPU
        ctx.check()
        setup_s.append(time.perf_counter() - t_setup)
    train_s = None
    if learned_ready:  # a network for this equation of state (Gamma 13/9)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        learned.train(ctx, p, n=int(args.train_pairs), opts=__import__("phoebus_gb300").abi.default_train_opts(
            epochs=args.train_epochs), device=dev)
        torch.cuda.synchronize()
        train_s = time.perf_counter() - t0
    from phoebus_gb300.fluid import MeshRK2

    rk = MeshRK2(ctx, p, mesh, blocks)
    dt = 0.5 * rk.estimate_dt(False)

    def step(batched, lrn):
        rk.step(dt, learned=lrn, batched=batched)

    zones = mesh.n[0] * mesh.n[1] * mesh.n[2]
    # prims, cons and the second-stage buffers (their ghosts feed the first
    # con2prim of a stage)
    snap = [(b["prim"].clone(), b["cons"].clone(), s2.clone()) for b, s2 in zip(blocks, rk.seconds)]

    def restore():
        for b, s2, (pr, co, sc) in zip(blocks, rk.seconds, snap):
            b["prim"].copy_(pr)
            b["cons"].copy_(co)
            s2.copy_(sc)

    k = args.torus_steps
    arms = [("batched", lambda: step(True, False), k)]
    if learned_ready:
        arms.append(("learned_batched", lambda: step(True, True), k))
    stream = torch.cuda.current_stream()
    med, per_round = _timed_rounds(arms, restore, args.section_rounds, stream)
    plain, _ = _timed_rounds([("plain_per_block", lambda: step(False, False), k)], restore, 1, stream)
    med.update(plain)
    per_round.update({"plain_per_block": [plain["plain_per_block"]]})
    res = {}
    for name in ["plain_per_block"] + [a[0] for a in arms]:
        res[name] = {"zone_updates_per_s": zones / (med[name] * 1e-3), "ms_per_step": med[name], "steps": k,
                     "rounds_ms": per_round[name]}
    fns = {"plain_per_block": (False, False), "batched": (True, False), "learned_batched": (True, True)}
    for name in res:
        restore()
        ctx.c2p_stats(reset=True)
        step(*fns[name])
        st = ctx.c2p_stats(reset=True)
        res[name].update({"c2p_iterations_per_zone": st["iterations"] / max(st["zones"], 1),
                          "c2p_residual_evals_per_zone": st["residual_evals"] / max(st["zones"], 1),
                          "c2p_failures": st["failures"]})
        if fns[name][1]:
            res[name]["c2p_learned_accepted_frac"] = st["learned_accepted"] / max(st["zones"], 1)
    ctx.check()
    nan = sum(int(torch.isnan(b["prim"][0][b.isl()]).sum()) for b in blocks)
    out = {"workload": f"FM torus on a {args.torus_n}^3 FMKS Kerr-Schild mesh (a 0.9375), "
                       f"{mesh.nblocks} uneven blocks, edges {mesh.lens}, WENO5-Z + HLL, Gamma 13/9, floors, "
                       "gr_outflow X1/X2 (bc_vars primitive, outer-X1 inflow check, FixFluxes), periodic X3",
           "interior_zones": zones, **res,
           "inputs": "every arm from the same snapshot of the initialised state; batched arms interleaved over "
                     f"{args.section_rounds} rounds of {k} steps, median round",
           "nan_interior_rho": nan, "field_factor": info["field_factor"], "training_seconds": train_s,
           "setup_seconds": setup_s[1], "setup_seconds_first_call": setup_s[0]}
    if "learned_batched" in res:
        out["learned_batched_over_plain"] = (res["learned_batched"]["zone_updates_per_s"] /
                                             res["plain_per_block"]["zone_updates_per_s"])
        out["learned_over_batched"] = (res["learned_batched"]["zone_updates_per_s"] /
                                       res["batched"]["zone_updates_per_s"])
    out["batched_over_plain"] = res["batched"]["zone_updates_per_s"] / res["plain_per_block"]["zone_updates_per_s"]
    del blocks, rk, snap
    torch.cuda.empty_cache()
    return out


def bench_m1(ctx, args, dev):
    """Radiation M1 moments (phx_radiation.h): an m1_n^3 periodic Minkowski
    block in the regime of the radiation_diffusion regression (gray
    scattering, optical depth 2 per zone, uniform fluid velocity 0.3 c, weak
    absorption), linear reconstruction.  RK2 steps of phx_rad_stage (opacities,
    fluxes, update, con2prim, implicit source, ghost exchange, con2prim) plus
    the radiation timestep estimate, timed with CUDA events; the per-task
    split is a separate pass with events around each task.  The oracle times
    the same step on an m1_cpu_n^3 sample on all host cores."""
    import numpy as np
    import torch

    from phoebus_gb300 import abi, radiation

    rc = radiation.RadiationContext(ctx)
    hb, par, rpar = radiation.radiation_pulse_3d(n=args.m1_n)
    p, rp = abi.default_params(**par), abi.default_rad_params(**rpar)
    db = hb.to_device(dev)
    del hb
    rc.MomentPrim2Con(rp, p, db)
    rc.Initialize(rp, p, db)
    rc.MomentCalculateOpacities(rp, p, db)
    dt = rc.EstimateTimestepBlock(rp, p, db)
    buf = torch.zeros_like(db["rcons"])
    dt_dev = torch.empty(1, dtype=torch.float64, device=dev)

    def step():
        rc.rk2_step(rp, p, db, buf, dt)
        rc.EstimateTimestepBlock(rp, p, db, out=dt_dev)

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.m1_steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.m1_steps
    zones = args.m1_n ** 3
    # per-task split of one stage (same launches as phx_rad_stage)
    base, out = db["rcons"].clone(), buf
    tasks = [("opacities", lambda: rc.MomentCalculateOpacities(rp, p, db)),
             ("fluxes", lambda: rc.CalculateFluxes(rp, p, db)),
             ("update", lambda: rc.Update(rp, db, base, out, 1.0, dt)),
             ("con2prim_interior", lambda: rc.MomentCon2Prim(rp, p, db, *db.interior())),  # no c2p fixup
             ("fluid_source", lambda: rc.MomentFluidSource(rp, p, db, dt)),
             ("ghost_exchange", lambda: rc.FillGhostsPeriodic(db)),
             ("con2prim_entire", lambda: rc.MomentCon2Prim(rp, p, db))]
    split = {}
    for name, fn in tasks:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        split[name] = a.elapsed_time(b)
    ctx.check()
    # FP64 rate of the flux kernel: ncu's FP64 operation count per face (the
    # production build, profiles/m1_fp64_per_unit.json) over the event time
    fp64 = None
    prof = ROOT / "profiles" / "m1_fp64_per_unit.json"
    if prof.exists():
        cnt = json.loads(prof.read_text())
        faces = 3 * args.m1_n * args.m1_n * (args.m1_n + 1)
        peak = ctx.probe_fp64_peak()
        ach = faces * cnt["flux_flops_per_face"] / (split["fluxes"] * 1e-3)
        inst = faces * cnt["flux_fp64_instructions_per_face"] / (split["fluxes"] * 1e-3)
        fp64 = {"kernel": "rad::k_fluxes (x1/x2/x3)", "achieved_tflops": ach / 1e12, "peak_tflops": peak / 1e12,
                "frac": ach / peak, "issue_frac": inst / (peak / 2.0),
                "flops_source": "ncu dadd + dmul + 2 dfma per face, 96^3 capture (profiles/m1_fp64_per_unit.json)",
                "peak_source": "measured in-process (phx_probe_fp64_peak)"}
    J = db["rprim"][abi.RJ][db.isl()]
    res = {"workload": f"M1 radiation, {args.m1_n}^3 periodic Minkowski block, gray scattering kappa dx = 2, "
                       "kappa_a = 1, fluid u = W (0.3, 0, 0), Gaussian J pulse, linear reconstruction; one RK2 "
                       "step (2 stages + timestep estimate) per step",
           "zone_updates_per_s": zones / (ms * 1e-3), "ms_per_step": ms, "steps": args.m1_steps,
           "stage_split_ms": split, "fp64": fp64, "nan_J": int(torch.isnan(J).sum()),
           "c2p_fail_zones": int((db["rprim"][abi.RFAIL][db.isl()] != 1.0).sum()),
           "gpu_launches_per_step": 2 * (4 + 3 + 2 + 1) + 3}
    del db, buf, base
    torch.cuda.empty_cache()
    if not args.no_cpu:
        from oracle.oracle import RadOracle

        os.environ["OMP_NUM_THREADS"] = str(os.cpu_count() or 1)
        o = RadOracle(tuned=True)
        hb, par, rpar = radiation.radiation_pulse_3d(n=args.m1_cpu_n)
        p, rp = abi.default_params(**par), abi.default_rad_params(**rpar)
        o.MomentPrim2Con(rp, p, hb)
        o.Initialize(rp, p, hb)
        o.MomentCalculateOpacities(rp, p, hb)
        hdt = o.EstimateTimestepBlock(rp, p, hb)
        hbuf = np.zeros_like(hb["rcons"])
        o.rk2_step(rp, p, hb, hbuf, hdt)
        times = []
        for _ in range(3):
            t0 = time.perf_counter()
            o.rk2_step(rp, p, hb, hbuf, hdt)
            o.EstimateTimestepBlock(rp, p, hb)
            times.append(time.perf_counter() - t0)
        t = min(times)
        res["cpu_baseline"] = {"value": args.m1_cpu_n ** 3 / t, "unit": UNIT, "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": f"oracle timing build, RK2 step on a {args.m1_cpu_n}^3 sample of the "
                                                         f"same state ({t:.2f} s/step)"}
        res["gpu_over_cpu"] = res["zone_updates_per_s"] / res["cpu_baseline"]["value"]
    return res


def cpu_model():
    """The host CPU's model name and logical core count."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() in ("Model name", "Vendor ID") and ":" in line:
                name = line.split(":", 1)[1].strip()
                if line.startswith("Model name"):
                    break
    except Exception:
        pass
    import platform

    return {"model": name or platform.processor() or "unknown", "arch": platform.machine(),
            "logical_cores": os.cpu_count() or 1}


def workload_config(args, ws):
    """The config object both arms print (same workload, same keys)."""
    n = args.n
    return {"workload": f"shear layer {n}^3 single block, Minkowski, Gamma 5/3, WENO5-Z + HLL, MHD, periodic; one "
                        "RK2 timestep (2 stages + timestep estimate) per step",
            "n": n, "ng": 4, "rk_stages_per_step": 2,
            "l2": "inputs larger than L2 (state ~%.1f GB)" % ((n + 8) ** 3 * 60 * 8 / 1e9),
            "parallelism": f"replicas x{ws}"}


def cpu_step_timer(n, threads, steps, warmup):
    """The oracle's timing build (-O3, contraction on) advancing an n^3 block
    of the shear layer by RK2 steps with the face-speed timestep estimate, on
    threads host threads; returns (seconds per step over `steps` timed steps,
    the per-step times)."""
    import numpy as np

    from oracle.oracle import Oracle
    from phoebus_gb300 import abi, states

    os.environ["OMP_NUM_THREADS"] = str(threads)
    o = Oracle(tuned=True)
    hb, par = states.kelvin_helmholtz(n=n)
    p = abi.default_params(**par)
    o.Initialize(p, hb)
    dt = 0.5 * o.EstimateTimestepBlock(p, hb, False)
    cs = np.zeros_like(hb["cons"])
    for _ in range(warmup):
        o.rk2_step(p, hb, cs, dt)
        o.EstimateTimestepBlock(p, hb, True)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        o.rk2_step(p, hb, cs, dt)
        o.EstimateTimestepBlock(p, hb, True)
        times.append(time.perf_counter() - t0)
    return sum(times) / len(times), times


def run_reference(args, ws, rank):
    """The reference's CPU path (the oracle port, timing build) on all host
    cores, on the same workload: the n^3 block itself (--ref-n 0), one RK2
    step + timestep estimate per bench step."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = args.ref_n or args.n
    t_step, _ = cpu_step_timer(n, threads, args.steps, args.warmup)
    v = n ** 3 / t_step
    cfg = workload_config(args, ws)
    sample = (f"the {n}^3 block itself" if n == args.n else f"{n}^3 sample of the {args.n}^3 shear layer") + \
             ", one RK2 step per bench step"
    if n != args.n:
        cfg["workload"] += f" (reference CPU path on a {n}^3 sample)"
        cfg["sample_n"] = n
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_step,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": cfg,
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                            "build": "oracle timing build: g++ -O3 -ffp-contract=fast -fno-math-errno "
                                     "-funroll-loops -fopenmp", "cpu": cpu_model()},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def _sig(x, d=4):
    """x rounded to d significant digits (compact summary numbers)."""
    if x is None or not isinstance(x, (int, float)):
        return x
    if x == 0 or x != x:
        return x
    import math

    return round(x, -int(math.floor(math.log10(abs(x)))) + d - 1)


def section_summary(fp64, c2p, batched, torus_res, m1):
    """The sections' headline numbers, short enough for the last line."""
    g = lambda d, *k: _sig(_dig(d, *k))  # noqa: E731
    out = {}
    if fp64:
        out["flux_fp64"] = {"tflops": g(fp64, "achieved_tflops"), "frac_of_probe": g(fp64, "frac"),
                            "issue_frac": g(fp64, "issue_frac")}
    if c2p:
        out["c2p_zones_per_s"] = {"plain": g(c2p, "plain", "zones_per_s"), "learned": g(c2p, "learned", "zones_per_s"),
                                  "ratio": g(c2p, "learned_over_plain"),
                                  "iters": [g(c2p, "plain", "iterations_per_zone"),
                                            g(c2p, "learned", "iterations_per_zone")],
                                  "accepted": g(c2p, "learned", "learned_accepted_frac"),
                                  "train_pairs": g(c2p, "training", "pairs")}
    if batched:
        out["batched_zone_updates_per_s"] = {
            "per_block": g(batched, "per_block", "zone_updates_per_s"),
            "batched": g(batched, "batched", "zone_updates_per_s"),
            "learned_batched": g(batched, "batched_learned", "zone_updates_per_s"),
            "learned_over_batched": g(batched, "learned_over_batched")}
    if torus_res:
        out["torus_zone_updates_per_s"] = {
            "plain": g(torus_res, "plain_per_block", "zone_updates_per_s"),
            "batched": g(torus_res, "batched", "zone_updates_per_s"),
            "learned_batched": g(torus_res, "learned_batched", "zone_updates_per_s"),
            "learned_over_batched": g(torus_res, "learned_over_batched")}
    if m1:
        out["m1_zone_updates_per_s"] = {"gpu": g(m1, "zone_updates_per_s"), "cpu": g(m1, "cpu_baseline", "value"),
                                        "flux_fp64_frac": g(m1, "fp64", "frac")}
    return out


def _dig(d, *keys):
    for k in keys:
        if not isinstance(d, dict) or k not in d:
            return None
        d = d[k]
    return d


def main():
    args = parse()
    ws, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    import numpy as np
    import torch

    from phoebus_gb300 import abi, states
    from phoebus_gb300.fluid import FluidContext

    dev = f"cuda:{local}"
    torch.cuda.set_device(local)
    if args.m1_only:
        ctx = FluidContext(local, exact=args.exact)
        if rank == 0:
            print(json.dumps({"m1": bench_m1(ctx, args, dev)}), flush=True)
        ctx.close()
        return
    n = args.n
    hb, par = states.kelvin_helmholtz(n=n)
    p = abi.default_params(**par)
    db = hb.to_device(dev)
    ctx = FluidContext(local, exact=args.exact)
    stream = torch.cuda.current_stream()
    ctx.Initialize(p, db)
    dt = 0.5 * ctx.EstimateTimestepBlock(p, db, False).item()
    base = db["cons"]
    second = torch.zeros_like(base)
    dt_out = torch.zeros(1, dtype=torch.float64, device=dev)

    def step(block):
        b0 = block["cons"]
        ctx.Stage(p, block, b0, second, 1.0, dt)
        block.arrays["cons"] = second
        ctx.Stage(p, block, b0, b0, 0.5, dt)
        block.arrays["cons"] = b0
        ctx.EstimateTimestepBlock(p, block, True, out=dt_out)

    for _ in range(args.warmup):
        step(db)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier(ws)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step(db)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ws, ms, dev)
    zones = n ** 3
    value = ws * zones / (ms * 1e-3)

    # dominant kernels: CalculateFluxes (three launches), timed live
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    torch.cuda.synchronize()
    f0.record(stream)
    for _ in range(reps):
        ctx.CalculateFluxes(p, db)
    f1.record(stream)
    torch.cuda.synchronize()
    flux_ms = f0.elapsed_time(f1) / reps
    hbm_peak, peak_src = measured_peaks()
    fb = flux_bytes(n, exact=args.exact)
    achieved = fb / (flux_ms * 1e-3) / 1e9
    fp64_peak = ctx.probe_fp64_peak()
    prof = ROOT / "profiles" / "flux_fp64_per_zone.json"
    fp64 = None
    if prof.exists():
        d = json.loads(prof.read_text())
        flops = d["fp64_flops_per_call_per_zone"] * zones
        fp64 = {"achieved_tflops": flops / (flux_ms * 1e-3) / 1e12, "peak_tflops": fp64_peak / 1e12,
                "frac": flops / (flux_ms * 1e-3) / fp64_peak, "flops_source": d["source"],
                "peak_source": "measured in-process (phx_probe_fp64_peak)"}
        if "fp64_instructions_per_call_per_zone" in d:
            # the probe issues DFMAs only (2 flops each): its instruction rate is peak / 2.  A kernel
            # with DADD/DMUL in its mix reaches frac < 1 at the full issue rate; issue_frac is the
            # FP64 instruction rate against the probe's.
            inst = d["fp64_instructions_per_call_per_zone"] * zones
            fp64["issue_frac"] = inst / (flux_ms * 1e-3) / (fp64_peak / 2.0)
            fp64["instructions_source"] = d["instructions_source"]
    traffic = None
    tf = ROOT / "profiles" / "flux_dram_traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get("bytes_per_call_scaled")

    # end to end through the C ABI with pinned host buffers.  Every step copies
    # its inputs (prims + cons) in and its result (prims + cons) out; the copies
    # run on two copy streams against a double-buffered device state, so the
    # H2D of step k+1 and the D2H of step k-1 overlap step k.
    e2e = None
    if not args.no_e2e:
        from phoebus_gb300.block import Block

        h_prim = torch.empty(db["prim"].shape, dtype=torch.float64, pin_memory=True)
        h_cons = torch.empty(db["cons"].shape, dtype=torch.float64, pin_memory=True)
        h_prim.copy_(db["prim"])
        h_cons.copy_(db["cons"])
        o_prim = torch.empty_like(h_prim).pin_memory()
        o_cons = torch.empty_like(h_cons).pin_memory()
        db2 = Block(db.nx, db.ng, db.ndim, db.xmin, db.dx, backend="torch", device=dev,
                    arrays={k: torch.empty_like(v) for k, v in db.arrays.items()})
        second2 = torch.zeros_like(second)
        bufs = [(db, second), (db2, second2)]

        def step_on(block, sec):
            b0 = block["cons"]
            ctx.Stage(p, block, b0, sec, 1.0, dt)
            saved = block.arrays["cons"]
            block.arrays["cons"] = sec
            ctx.Stage(p, block, b0, b0, 0.5, dt)
            block.arrays["cons"] = saved
            ctx.EstimateTimestepBlock(p, block, True, out=dt_out)

        h2d_stream, d2h_stream = torch.cuda.Stream(), torch.cuda.Stream()
        for blk, sec in bufs:  # warm the second buffer's path once
            blk["prim"].copy_(h_prim)
            blk["cons"].copy_(h_cons)
            step_on(blk, sec)
        torch.cuda.synchronize()
        barrier(ws)
        free = [None, None]
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        h2d_stream.wait_stream(stream)
        d2h_stream.wait_stream(stream)
        for k in range(args.steps):
            blk, sec = bufs[k % 2]
            with torch.cuda.stream(h2d_stream):
                if free[k % 2] is not None:
                    h2d_stream.wait_event(free[k % 2])
                blk["prim"].copy_(h_prim, non_blocking=True)
                blk["cons"].copy_(h_cons, non_blocking=True)
                ready = torch.cuda.Event()
                ready.record(h2d_stream)
            stream.wait_event(ready)
            step_on(blk, sec)
            done = torch.cuda.Event()
            done.record(stream)
            with torch.cuda.stream(d2h_stream):
                d2h_stream.wait_event(done)
                o_prim.copy_(blk["prim"], non_blocking=True)
                o_cons.copy_(blk["cons"], non_blocking=True)
                f = torch.cuda.Event()
                f.record(d2h_stream)
                free[k % 2] = f
        stream.wait_stream(d2h_stream)
        g1.record(stream)
        torch.cuda.synchronize()
        barrier(ws)
        ems = max_over_ranks(ws, g0.elapsed_time(g1) / args.steps, dev)
        nb = (h_prim.numel() + h_cons.numel()) * 8
        e2e = {"value": ws * zones / (ems * 1e-3), "unit": UNIT, "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb,
               "ms_per_step": ems, "pipelining": "double-buffered; H2D of step k+1 and D2H of k-1 overlap step k"}
        del db2, second2
    ctx.check()
    c2p = None if args.no_c2p else bench_c2p(ctx, args, dev)
    batched = None if args.no_batched else bench_batched(ctx, args, dev, learned_ready=c2p is not None)
    torus_res = None if args.no_torus else bench_torus(ctx, args, dev, learned_ready=not args.no_c2p)
    m1_res = None if args.no_m1 else bench_m1(ctx, args, dev)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        t, _ = cpu_step_timer(args.cpu_n, threads, 3, 1)
        cpu = {"value": args.cpu_n ** 3 / t, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"oracle timing build, RK2 step on a {args.cpu_n}^3 sample of the same state "
                         f"({t:.2f} s/step, 3 steps after 1 warm-up)", "cpu": cpu_model()}

    if rank == 0:
        detail = {"fp64": fp64, "c2p": c2p, "batched": batched, "torus": torus_res, "m1": m1_res}
        print(json.dumps({"detail": detail}), flush=True)  # full sections, one line before the result
        cfg = workload_config(args, ws)
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg, "build": "exact" if args.exact else "production",
            "zone_stages_per_s": 2 * value,
            "roofline": {"bound": "hbm", "achieved": _sig(achieved, 6), "peak": hbm_peak, "unit": "GB/s",
                         "frac": _sig(achieved / hbm_peak, 6), "traffic": traffic, "kernel": "CalculateFluxes x1-x3",
                         "peak_source": peak_src, "algorithmic_bytes": fb, "launch_ms": _sig(flux_ms, 6),
                         "note": "FP64-bound; see sections.flux_fp64"},
            "sections": section_summary(fp64, c2p, batched, torus_res, m1_res),
            "cpu_baseline": cpu,
            "clocks": clocks,
            "e2e": e2e,
            "gpu_launches": args.steps * (2 * stage_launches(n) + LAUNCHES_DT),
        }
        print(json.dumps(out), flush=True)
    ctx.close()
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()

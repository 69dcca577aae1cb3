"""Benchmark of the ACSF + BPNN hot path on one GB300: the batching configuration C3.

Workload (C3): 20,000 periodic structures of 8-2,048 atoms (log-uniform, 7.4 M atoms), three
species, 168 ACSF features (72 radial + 96 angular after species expansion, cutoff 6 A),
per-species networks 168-64-64-1 tanh, energy targets.  Features are computed once per run,
as the reference does (prog/fortnet/prg_fnet/fortnet.F90:840-921), and reported separately.

One step = one training pass over every structure + the energies of every structure:
  batched form   one epoch of 256-structure mini-batches: per mini-batch forward, loss,
                 reverse pass and steepest-descent step, BF16 tensor-core GEMMs with FP32
                 accumulation, FP64 gradient sums and parameters, replayed as one CUDA graph;
                 then a tensor-core forward over every structure
  plain form     one L-BFGS iteration of the reference's nTrain loop on the whole dataset
                 (FP32 SIMT kernels, FP64 reductions and optimiser state), then a forward over
                 every structure
Metric: atoms/s = atoms in the dataset / step time.  `value` is the batched form with inputs
resident in HBM (L2 flushed between timed steps); `forms` gives both forms and their ratio,
and their energy errors against an FP64 evaluation of the same parameters.
`e2e`: the batched step through the public API from host coordinates: coordinates copied in,
featurisation, feature packing, the epoch and the energies, the loss and the energies copied
out, all inside the timed region.

--impl reference times the CPU restatement of the reference's own algorithm (the oracle:
neighbour list rebuilt per atom and G-function, per-atom network evaluation) with all host
threads on a bounded sample of the same workload: featurise + one L-BFGS iteration + energies.
"""

from __future__ import annotations

import argparse
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

METRIC = ("atoms/s train+predict (C3: one training epoch over every structure + energies; "
          "batched mixed-precision form)")
UNIT = "atoms/s"
L2_FLUSH_BYTES = 256 << 20
BATCH = 256  # structures per mini-batch (C3)


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if s[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def oracle_params(cfg, dims):
    """The reference's initial parameters (RANLUX lux 3 normalXavier, as TBpnn_init draws
    them), from the oracle's restatement."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    return O.Ranlux(cfg.seed).init_bpnn(dims, "tanh", len(cfg.atomic_numbers))


def featurise(ctx, zprec=None, weights=None):
    ctx.npairs = ctx.neighbors()
    ctx.acsf(download=False)
    return ctx.zscore(weights=weights, zprec=zprec)


def acsf_op_counts(funcs, species_frac):
    """Algorithmic work of the ACSF value pass in the moment form, from the G-function list:
    (FP32 operations per pair, per atom; ex2 operations per pair; bytes per pair, per atom).
    Per pair: the cutoff (one sine, 4 operations), every radial G2 whose list holds the pair
    (x = r - rs, x^2, the scale, the exponential, times fc, the sum: 5 operations and one ex2;
    a resolved function holds its species' share of the pairs), per angular eta class
    E = exp(-eta r^2) fc (2 operations, one ex2) and the 35 moment products and sums of degree
    <= 4 (70 operations), plus the 34 products building the monomials once.  Per atom: per
    (channel pair, eta class) the degree sums over the 35 monomials (3 operations each), per G5
    function the combination of its five degree sums (10).  HBM: the pair record (displacement
    and distance 16 B, neighbour 4 B, image and class 4 B) per pair; per atom the features (4 B
    each) and the moment cache (35 FP32 per list and eta class)."""
    rad = [f for f in funcs if f.radial]
    ang = [f for f in funcs if f.angular]
    def frac(z):
        return 1.0 if z == 0 else species_frac.get(z, 0.0)

    per_pair = 4.0 + sum(5.0 * frac(f.z1) for f in rad)
    ex2_pair = 1.0 + sum(frac(f.z1) for f in rad)
    per_atom = 0.0
    mom_bytes = 0.0
    if ang:
        etas = sorted({f.eta for f in ang})
        lists = sorted({f.z1 for f in ang} | {f.z2 for f in ang})
        chpairs = sorted({(min(f.z1, f.z2), max(f.z1, f.z2)) for f in ang})
        # a pair enters its species' list (and the all-atom list when one is used)
        share = sum(frac(z) for z in lists)
        per_pair += 34.0 + len(etas) * share * (2.0 + 70.0)
        ex2_pair += len(etas) * share
        per_atom = len(chpairs) * len(etas) * 35 * 3.0 + len(ang) * 10.0
        mom_bytes = 4.0 * 35 * len(lists) * len(etas)
    return per_pair, per_atom, ex2_pair, 24.0, 4.0 * len(funcs) + mom_bytes


def setup(args):
    from fortnet_gb300 import api, synthetic

    cfg = synthetic.CONFIGS[args.config]
    t0 = time.perf_counter()
    ds = synthetic.generate(cfg, nstruct=args.nstruct)
    gen_s = time.perf_counter() - t0
    funcs = synthetic.gfunctions(cfg)
    dims = synthetic.network_dims(cfg)
    ctx = api.Context(api.FP32)
    ctx.upload(ds)
    ctx.set_species(ds.species)
    ctx.set_gfunctions(funcs)
    zprec = featurise(ctx, weights=ds.weights)
    params = oracle_params(cfg, dims)
    ctx.set_network(dims, "tanh", params)
    ctx.set_targets(ds)
    ctx.optimizer_init("lbfgs", 1e-20, 1e-6, 1e4, memory=1000, linemin=True)
    ctx.batch_setup(args.batch)
    return ctx, ds, zprec, funcs, dims, params, gen_s


def plain_step(ctx):
    """The plain FP32 form: one full-batch L-BFGS iteration + energies of every atom."""
    ctx.train_iteration("mse")
    ctx.lib.fnetg_predict(ctx.h, None, None)


def batched_step(ctx, lr):
    """The batched mixed-precision form: one epoch of mini-batch steps + every energy."""
    ctx.batch_epoch("mse", lr, args_maxdisp(), want_loss=False)
    ctx.lib.fnetg_batch_predict(ctx.h, None, None)


def args_maxdisp():
    return 1e4


def e2e_step(ctx, zprec, coords_pinned, out_energy, out_loss, lr):
    """The batched step through the public API from host coordinates: coordinates uploaded
    from pinned memory, featurisation and feature packing, the epoch, the energies; the loss
    and the per-structure energies downloaded into pinned buffers."""
    ctx.update_coords(coords_pinned)
    featurise(ctx, zprec=zprec)
    ctx.batch_setup(BATCH)
    ctx.lib.fnetg_batch_epoch(ctx.h, 0, lr, args_maxdisp(), out_loss.ctypes.data)
    ctx.batch_predict(atomic=False, out_global=out_energy)


def timed(ctx, fn, steps, stream, flush, torch):
    """CUDA-event time of each step on the library's stream, L2 flushed between steps."""
    times = []
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return times


def energy_errors(ctx, ds, funcs, zprec, dims, nsample=64):
    """Per-structure energy errors of both forms against an FP64 evaluation of the same
    parameters, on the first structures of the dataset."""
    from fortnet_gb300 import api

    params = ctx.params()
    _, e_tc = ctx.batch_predict(atomic=False)
    ctx.lib.fnetg_batch_sync_params(ctx.h)
    _, e_32 = ctx.predict(atomic=False)
    k = min(nsample, ds.nstruct)
    sub_off = ds.atom_offsets[:k + 1]
    from fortnet_gb300.fnetdata import Dataset

    n = int(sub_off[-1])
    sub = Dataset(atom_offsets=sub_off, coords=ds.coords[:n], atnum=ds.atnum[:n],
                  species=ds.species[:n], periodic=ds.periodic[:k], latvecs=ds.latvecs[:k],
                  atomic_numbers=ds.atomic_numbers, weights=ds.weights[:k],
                  atomic_weights=ds.atomic_weights[:n], global_targets=ds.global_targets[:k],
                  atomic_targets=ds.atomic_targets[:n])
    with api.Context(api.FP64) as c:
        c.upload(sub)
        c.set_species(sub.species)
        c.set_gfunctions(funcs)
        c.acsf(download=False)
        c.zscore(zprec=zprec)
        c.set_network(dims, "tanh", params)
        at64, e_64 = c.predict(atomic=True)
    # relative to sum_i |o_i| of each structure: some structures' energies are small
    # differences of large atomic outputs, where |E| is not the scale of an error
    mag = np.add.reduceat(np.abs(at64[:, 0]), sub_off[:-1])
    nat = np.diff(sub_off).astype(np.float64)

    def stats(e):
        d = np.abs(e[:k, 0] - e_64[:k, 0])
        return {"max_rel": float(f"{np.max(d / mag):.3g}"),
                "median_rel": float(f"{np.median(d / mag):.3g}"),
                "rmse_per_atom": float(f"{np.sqrt(np.mean((d / nat) ** 2)):.3g}")}

    return {"structures": k, "metric": "|E - E64| / sum_i |o_i,64| per structure; RMSE of "
                                       "(E - E64) / atoms",
            "plain_fp32": stats(e_32), "batched_bf16": stats(e_tc)}


def featurise_roofline(ctx, ds, funcs, feat_prof, nfeat=2):
    """Rooflines of the featurisation stages, from their CUDA-event times over nfeat
    featurisations: the ACSF value pass against the device's measured FP32 and ex2 rates and
    HBM bandwidth, the neighbour search (its kernels together) against HBM (its pair records
    written once: 24 B per pair, plus positions read and cell-sorted)."""
    fp32_peak, ex2_peak, fp64_peak = ctx.probe_peaks()
    hbm, _, peak_kind = load_peaks()
    N, P = ds.ntot, float(ctx.npairs)
    zs, cnt = np.unique(ds.atnum, return_counts=True)
    frac = {int(z): float(c) / N for z, c in zip(zs, cnt)}
    fpp, fpa, epp, bpp, bpa = acsf_op_counts(funcs, frac)
    out = {"pairs": int(P), "peaks": {"fp32_tflops": round(fp32_peak, 1),
                                      "ex2_tops": round(ex2_peak, 2),
                                      "fp64_tflops": round(fp64_peak, 3), "hbm_gbs": hbm,
                                      "source": "fnetg_probe_peaks (FMA and ex2 loops, CUDA "
                                                "events) and MEASURED_PEAKS.json " + peak_kind}}
    ms, n = feat_prof["acsf"]
    if n:
        sec = ms / nfeat / 1e3
        fl = (P * fpp + N * fpa) / sec / 1e12
        ex = P * epp / sec / 1e12
        gb = (P * bpp + N * bpa) / sec / 1e9
        out["acsf"] = {"ms": round(ms / nfeat, 3),
                       "flop_per_pair": round(fpp, 1), "flop_per_atom": round(fpa, 1),
                       "ex2_per_pair": round(epp, 2),
                       "fp32": {"achieved": round(fl, 2), "peak": round(fp32_peak, 1),
                                "unit": "TFLOP/s", "frac": round(fl / fp32_peak, 4)},
                       "ex2": {"achieved": round(ex, 3), "peak": round(ex2_peak, 2),
                               "unit": "Top/s", "frac": round(ex / ex2_peak, 4)},
                       "hbm": {"achieved": round(gb, 1), "peak": hbm, "unit": "GB/s",
                               "frac": round(gb / hbm, 4)}}
    ms, n = feat_prof["neighbors"]
    if n:
        sec = ms / nfeat / 1e3
        gb = (P * 24.0 + N * 32.0) / sec / 1e9
        out["neighbors"] = {"ms": round(ms / nfeat, 3), "bytes_per_pair": 24,
                            "hbm": {"achieved": round(gb, 1), "peak": hbm, "unit": "GB/s",
                                    "frac": round(gb / hbm, 4)}}
    return out


def run_ours(args):
    from fortnet_gb300 import api

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # replicas only: barrier + max-over-ranks timing

        dist.init_process_group("gloo")
    import torch

    torch.cuda.set_device(local)
    ctx, ds, zprec, funcs, dims, params, gen_s = setup(args)
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    N = ds.ntot
    lr = args.lr
    # one-time featurisation (the reference computes features once per run), timed alone
    ctx.synchronize()
    ctx.profile(True)
    ctx.profile_reset()
    feat_ms = float(np.mean(timed(ctx, lambda: featurise(ctx, zprec=zprec), 2, stream, flush,
                                  torch)))
    feat_prof = {f: ctx.profile_read(f) for f in ("neighbors", "scan", "acsf", "zscore")}
    ctx.profile(False)
    feat_roof = featurise_roofline(ctx, ds, funcs, feat_prof)
    ctx.batch_setup(args.batch)
    # plain FP32 form, then the batched mixed-precision form (the headline); the warm-up of
    # the batched form captures the epoch graph and runs the autotuner.  The clock sampler
    # runs through both timed regions (a batched step lasts a few ms, shorter than the
    # sampling interval).
    for _ in range(args.warmup):
        plain_step(ctx)
    for _ in range(args.warmup):
        batched_step(ctx, lr)
    ctx.synchronize()
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        plain_ms = float(np.mean(timed(ctx, lambda: plain_step(ctx), args.plain_steps, stream,
                                       flush, torch)))
        for _ in range(2):
            batched_step(ctx, lr)  # the plain steps moved the parameters: images re-packed
        launches0 = ctx.launch_count()
        times = timed(ctx, lambda: batched_step(ctx, lr), args.steps, stream, flush, torch)
    torch.cuda.synchronize()
    launches = ctx.launch_count() - launches0
    ms_step = float(np.mean(times))
    if dist:
        t = torch.tensor([ms_step], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    value = N * world / (ms_step / 1e3)
    # per-kernel device times of one batched step, launched eagerly with CUDA events (the
    # profiled epoch runs the same kernels without the graph)
    ctx.profile(True)
    ctx.profile_reset()
    batched_step(ctx, lr)
    ctx.synchronize()
    fams = ["tc_forward", "tc_train", "tc_reduce", "tc_update", "tc_pack", "loss"]
    prof = {f: ctx.profile_read(f) for f in fams}
    ctx.profile(False)
    info = ctx.batch_info()
    errs = energy_errors(ctx, ds, funcs, zprec, dims)
    # ---- end to end through the public API with host buffers (pinned)
    coords = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    coords[:] = ds.coords
    energy = torch.empty((ds.nstruct, 1), dtype=torch.float64, pin_memory=True).numpy()
    loss = torch.empty(1, dtype=torch.float64, pin_memory=True).numpy()
    for _ in range(2):
        e2e_step(ctx, zprec, coords, energy, loss, lr)
    ctx.synchronize()
    t0 = time.perf_counter()
    esteps = max(2, min(args.steps, 5))
    for _ in range(esteps):
        e2e_step(ctx, zprec, coords, energy, loss, lr)
    ctx.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / esteps
    h2d = coords.nbytes
    d2h = energy.nbytes + loss.nbytes
    accuracy = accuracy_leg(args, ctx, ds, zprec, funcs, dims) if args.acc_epochs > 0 else None
    # ---- roofline of the dominant kernel of the step: algorithmic FLOPs (tensor pipe) and
    # algorithmic HBM bytes per launch against the measured peaks; the bound is the nearer roof
    hbm, bf16_peak, peak_kind = load_peaks()
    nf, h1, h2 = dims[0], dims[1], dims[2]
    fwd_flop = 2 * (nf * h1 + h1 * h2 + h2)          # per atom, one forward
    train_flop = 2 * fwd_flop + 2 * h1 * h2            # forward again, delta_1, weight gradients
    xrow = 2 * (((nf + 1) + 15) // 16 * 16)            # BF16 feature bytes per atom
    per_atom = {"tc_forward": (fwd_flop, xrow + 8), "tc_train": (train_flop, xrow + 8)}
    dom = max((f for f in fams if prof[f][1] > 0), key=lambda f: prof[f][0])
    roof = {"kernel": dom, "launch_ms": round(prof[dom][0] / max(prof[dom][1], 1), 5),
            "launches_per_step": int(prof[dom][1])}
    if dom in per_atom:
        # every tensor-core launch of the step covers one mini-batch; tc_forward also runs once
        # over every atom (the prediction): atoms processed per step = N x launches' share
        atoms_total = N * (2 if dom == "tc_forward" else 1)
        secs = prof[dom][0] / 1e3
        fl, by = per_atom[dom]
        tflops = atoms_total * fl / secs / 1e12
        gbs = atoms_total * by / secs / 1e9
        tensor = {"achieved": round(tflops, 2), "peak": bf16_peak, "unit": "TFLOP/s",
                  "frac": round(tflops / bf16_peak, 4)}
        mem = {"achieved": round(gbs, 1), "peak": hbm, "unit": "GB/s", "frac": round(gbs / hbm, 4)}
        best = ("tensor", tensor) if tensor["frac"] >= mem["frac"] else ("hbm", mem)
        roof.update({"bound": best[0], **best[1], "tensor_roof": tensor, "hbm_roof": mem,
                     "algorithmic_flop_per_atom": fl, "algorithmic_bytes_per_atom": by,
                     "peak_source": peak_kind})
    else:
        roof.update({"bound": "latency", "note": "a small reduction / update kernel dominates"})
    atoms_per_launch = (N * (2 if dom == "tc_forward" else 1)) / max(prof[dom][1], 1)
    traffic, traffic_src = profiled_traffic(dom, args.config, atoms_per_launch)
    roof["traffic"] = traffic
    roof["traffic_source"] = traffic_src
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic (seeded C3 generator: dense-liquid cells, Morse energy targets)",
        "config": {"workload": f"{args.config}: {ds.nstruct} structures, {N} atoms, "
                               f"{dims[0]} features, net {'-'.join(map(str, dims))}, mini-batches "
                               f"of {args.batch} structures ({info['batches']} per epoch, "
                               f"{info['tiles']} tiles of 128 atoms)",
                   "l2": "flushed between timed steps (256 MiB write)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "forms": {
            "batched_bf16": {"atoms_per_s": round(value / world, 1), "ms_per_step": round(ms_step, 3)},
            "plain_fp32": {"atoms_per_s": round(N / (plain_ms / 1e3), 1),
                           "ms_per_step": round(plain_ms, 3)},
            "ratio": round(plain_ms / ms_step, 2),
            "errors_vs_fp64": errs,
            "featurise_ms": round(feat_ms, 2),
            "featurise_atoms_per_s": round(N / (feat_ms / 1e3), 1),
            "featurise_kernels_ms": {f: round(v[0] / 2, 3) for f, v in feat_prof.items() if v[1]},
            "featurise_roofline": feat_roof,
            "dataset_generation_s": round(gen_s, 1),
        },
        "accuracy": accuracy,
        "e2e": {"value": round(N / (e2e_ms / 1e3), 1), "unit": UNIT,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "kernels_ms_per_step": {f: round(prof[f][0], 4) for f in fams if prof[f][1] > 0},
        "kernel_launches_per_step": {f: int(prof[f][1]) for f in fams if prof[f][1] > 0},
        "autotuned_ctas": {"forward": info["ctas_forward"], "train": info["ctas_train"]},
        "clocks": clk.summary(),
    }
    if rank == 0 and (args.c4_iters > 0 or args.serve_requests > 0 or not args.no_lbfgs):
        ctx.close()
    if args.c4_iters > 0 and rank == 0:
        out["precision_c4"] = precision_leg(args)
    if not args.no_lbfgs and rank == 0:
        out["lbfgs_full_history"] = lbfgs_leg(args)
    if args.serve_requests > 0 and rank == 0:
        out["serving"] = serving_leg(args)
    if not args.no_cpu_baseline and rank == 0 and world == 1:
        out["cpu_baseline"] = cpu_baseline(args, threads=1)
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def accuracy_leg(args, ctx, ds, zprec, funcs, dims):
    """Test-set accuracy of the two forms on C3.  Both train from the same well-conditioned
    initial weights (N(0, 1/fan_in)) on the whole C3 dataset: the batched form for
    args.acc_epochs epochs at each learning rate of a small sweep, the plain form (full-batch
    L-BFGS with line search) for the wall time of the batched form's best run.  A held-out
    set of C3 structures (generator seed + 7, Morse energies and forces) is evaluated with the
    plain FP32 kernels (energies, analytical forces) and with the BF16 tensor-core forward
    (energies): RMSE of the energy per atom and of the force components, in the targets'
    units (Hartree, Hartree/Bohr)."""
    import dataclasses

    from fortnet_gb300 import api, synthetic

    cfg = synthetic.CONFIGS[args.config]
    test = synthetic.generate(dataclasses.replace(cfg, seed=cfg.seed + 7),
                              nstruct=args.acc_test_structs, forces=True)
    params0 = synthetic.normal_params(dims, len(cfg.atomic_numbers), cfg.seed)
    nat = np.diff(test.atom_offsets).astype(np.float64)
    et = test.global_targets[:, 0]
    ft = test.meta["forces"]
    tc = api.Context(api.FP32)
    tc.upload(test)
    tc.set_species(test.species)
    tc.set_gfunctions(funcs)
    featurise(tc, zprec=zprec)
    tc.set_network(dims, "tanh", params0)
    tc.set_targets(test)

    def evaluate(params):
        tc.set_network(dims, "tanh", params)
        tc.batch_setup(BATCH)
        _, e32 = tc.predict(atomic=False)
        f32 = tc.forces()[:, 0, :]
        _, e16 = tc.batch_predict(atomic=False)
        r = lambda e: float(f"{np.sqrt(np.mean(((e[:, 0] - et) / nat) ** 2)):.4g}")
        return {"energy_rmse_per_atom_fp32": r(e32), "energy_rmse_per_atom_bf16": r(e16),
                "force_rmse_fp32": float(f"{np.sqrt(np.mean((f32 - ft) ** 2)):.4g}")}

    out = {"test_set": f"{test.nstruct} held-out {args.config} structures, {test.ntot} atoms",
           "init": "N(0, 1/fan_in) weights, N(0, 0.01) biases",
           "initial": evaluate(params0), "batched_sweep": {}}
    best = None
    for lr in args.acc_lrs:
        ctx.set_network(dims, "tanh", params0)
        ctx.batch_setup(args.batch)
        ctx.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.acc_epochs):
            ctx.batch_epoch("mse", lr, args_maxdisp(), want_loss=False)
        ctx.synchronize()
        secs = time.perf_counter() - t0
        res = evaluate(ctx.params())
        res["seconds"] = round(secs, 3)
        out["batched_sweep"][f"{lr:g}"] = res
        if np.isfinite(res["energy_rmse_per_atom_fp32"]) and (
                best is None or res["energy_rmse_per_atom_fp32"] < best[1]["energy_rmse_per_atom_fp32"]):
            best = (lr, res)
    out["batched"] = {"learning_rate": best[0], "epochs": args.acc_epochs, **best[1]}
    # the plain form for the same wall time
    ctx.set_network(dims, "tanh", params0)
    ctx.optimizer_init("lbfgs", 1e-20, 1e-6, 1e4, memory=1000, linemin=True)
    ctx.synchronize()
    t0 = time.perf_counter()
    iters = 0
    while time.perf_counter() - t0 < best[1]["seconds"]:
        ctx.train_iteration("mse")
        ctx.synchronize()
        iters += 1
    secs = time.perf_counter() - t0
    out["plain"] = {"iterations": iters, "seconds": round(secs, 3), **evaluate(ctx.params())}
    tc.close()
    return out


def profiled_traffic(kernel, config, atoms_per_launch):
    """DRAM bytes per launch of `kernel` from the committed ncu summary of this configuration:
    the bytes per atom measured on a capture of the same kernel and mini-batch size, times the
    atoms one launch of this run processes."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_kernel_{config}.md")
    if not os.path.exists(path):
        return None, None
    with open(path) as fh:
        for line in fh:
            if line.startswith("dram_bytes_per_atom:"):
                per_atom = float(line.split(":", 1)[1])
                return int(per_atom * atoms_per_launch), os.path.relpath(path, ROOT)
    return None, None


def c4_model(args):
    """The C4 model of the serving stream: 66-64-64-1 tanh networks trained with the precision
    form's loss, energies + 0.1 x force MSE against Morse targets, by L-BFGS on a C4 training
    sample, from well-conditioned initial weights (N(0, 1/fan_in)); the reference's
    normalXavier draw saturates the tanh units and stays saturated through training.  Returns
    the parameters, the training sample's z-score statistics and the training record."""
    from fortnet_gb300 import api, synthetic

    cfg = synthetic.CONFIGS["C4"]
    ds = synthetic.generate(cfg, nstruct=args.model_structs, forces=True)
    funcs = synthetic.gfunctions(cfg)
    dims = synthetic.network_dims(cfg)
    params = synthetic.normal_params(dims, len(cfg.atomic_numbers), cfg.seed)
    with api.Context(api.FP32) as c:
        c.upload(ds)
        c.set_species(ds.species)
        c.set_gfunctions(funcs)
        zprec = featurise(c, weights=ds.weights)
        c.set_network(dims, "tanh", params)
        c.set_targets(ds)
        c.set_force_targets(0.1, ds.meta["forces"])
        c.optimizer_init("lbfgs", 1e-20, 1e-6, 1e4, memory=1000, linemin=True)
        t0 = time.perf_counter()
        first = None
        for _ in range(args.model_iters):
            c.train_iteration("mse")
            if first is None:
                first = c.last_losses()
        last = c.last_losses()
        secs = time.perf_counter() - t0
        params = c.params()
    rec = {"init": "N(0, 1/fan_in) weights, N(0, 0.01) biases (seed 1004)",
           "structures": ds.nstruct, "atoms": ds.ntot, "iterations": args.model_iters,
           "loss_energy": [float(f"{first[0]:.4g}"), float(f"{last[0]:.4g}")],
           "loss_forces": [float(f"{first[1]:.4g}"), float(f"{last[1]:.4g}")],
           "seconds": round(secs, 2)}
    return params, zprec, funcs, dims, rec


def precision_leg(args):
    """The precision form on C4 (5,000 structures of 100-500 atoms, three species, 66 features,
    66-64-64-1 tanh, cutoff 6.5 A): training iterations of the loss energies + 0.1 x force MSE
    (forward, analytical forces, dG/dR contraction, reverse pass with tangents, FP64 gradient
    reduction, L-BFGS with FP64 state) with the network passes in FP32 SIMT kernels and on the
    tensor cores (BF16 operands, FP32 accumulation); atoms/s per iteration, and the results'
    errors against an FP64 run of the same kernels (energies, forces, gradient).  Initial
    weights N(0, 1/fan_in) (the served C4 model's)."""
    from fortnet_gb300 import api, synthetic
    from fortnet_gb300.fnetdata import Dataset

    cfg = synthetic.CONFIGS["C4"]
    ds = synthetic.generate(cfg, nstruct=args.c4_structs, forces=True)
    funcs = synthetic.gfunctions(cfg)
    dims = synthetic.network_dims(cfg)
    params = synthetic.normal_params(dims, len(cfg.atomic_numbers), cfg.seed)
    out = {"workload": f"C4: {ds.nstruct} structures, {ds.ntot} atoms, {dims[0]} features, net "
                       f"{'-'.join(map(str, dims))}, loss E + 0.1 F-MSE, L-BFGS"}
    fams = ["mlp_forward", "mlp_jacobian", "forces", "features_jvp", "force_loss_backward",
            "force_loss", "loss", "reduce", "optimizer", "params", "tc_jacobian", "tc_tangent",
            "tc_reduce", "tc_pack"]
    for form in ("plain_fp32", "bf16_tensor_cores"):
        with api.Context(api.FP32) as c:
            c.upload(ds)
            c.set_species(ds.species)
            c.set_gfunctions(funcs)
            zprec = featurise(c, weights=ds.weights)
            c.set_network(dims, "tanh", params)
            c.set_targets(ds)
            c.set_force_targets(0.1, ds.meta["forces"])
            if form == "bf16_tensor_cores":
                c.batch_setup(args.batch)
                c.batch_train_bf16(True)
            c.optimizer_init("lbfgs", 1e-20, 1e-6, 1e4, memory=1000, linemin=True)
            for _ in range(2):
                c.train_iteration("mse")
            c.synchronize()
            c.profile(True)
            c.profile_reset()
            t0 = time.perf_counter()
            for _ in range(args.c4_iters):
                c.train_iteration("mse")
            c.synchronize()
            dt = (time.perf_counter() - t0) / args.c4_iters
            prof = {f: c.profile_read(f) for f in fams}
            c.profile(False)
            params_now = c.params()
            out[form] = {"atoms_per_s": round(ds.ntot / dt, 1),
                         "ms_per_iteration": round(dt * 1e3, 3), "iterations": args.c4_iters,
                         "kernels_ms_per_iteration": {f: round(v[0] / args.c4_iters, 4)
                                                      for f, v in prof.items() if v[1]},
                         "losses": dict(zip(("energy", "forces"), c.last_losses()))}
    # FP32 against FP64 on the first structures, same parameters
    k = min(32, ds.nstruct)
    n = int(ds.atom_offsets[k])
    sub = Dataset(atom_offsets=ds.atom_offsets[:k + 1], coords=ds.coords[:n], atnum=ds.atnum[:n],
                  species=ds.species[:n], periodic=ds.periodic[:k], latvecs=ds.latvecs[:k],
                  atomic_numbers=ds.atomic_numbers, weights=ds.weights[:k],
                  atomic_weights=ds.atomic_weights[:n], global_targets=ds.global_targets[:k],
                  atomic_targets=ds.atomic_targets[:n])
    res = {}
    for prec in (api.FP32, api.FP64):
        with api.Context(prec) as c:
            c.upload(sub)
            c.set_species(sub.species)
            c.set_gfunctions(funcs)
            featurise(c, zprec=zprec)
            c.set_network(dims, "tanh", params_now)
            c.set_targets(sub)
            c.set_force_targets(0.1, ds.meta["forces"][:n])
            at, e = c.predict(atomic=True)
            F = c.forces()[:, 0, :]
            g, _, _ = c.train_gradients("mse")
            res[prec] = (e[:, 0], F, g, at[:, 0])
    e32, F32, g32, _ = res[api.FP32]
    e64, F64, g64, at64 = res[api.FP64]
    off = sub.atom_offsets
    # relative to sum_i |o_i| of the structure (energies that are small differences of large
    # atomic outputs are not the scale of their rounding)
    mag = np.add.reduceat(np.abs(at64), off[:-1])
    f_err = max(float(np.max(np.abs(F32[off[s]:off[s + 1]] - F64[off[s]:off[s + 1]]))
                      / np.max(np.abs(F64[off[s]:off[s + 1]]))) for s in range(k))
    g_err = max(float(np.linalg.norm(g32[s] - g64[s]) / np.linalg.norm(g64[s]))
                for s in range(g64.shape[0]))
    out["errors_fp32_vs_fp64"] = {
        "structures": k, "energy_rel": float(f"{np.max(np.abs(e32 - e64) / mag):.3g}"),
        "energy_metric": "|E32 - E64| / sum_i |o_i,64| per structure",
        "force_rel_of_max": float(f"{f_err:.3g}"), "gradient_rel": float(f"{g_err:.3g}"),
        "parameters": "after the timed tensor-core iterations"}
    # the tensor-core gradient against the FP64 one at the same parameters
    with api.Context(api.FP32) as c:
        c.upload(sub)
        c.set_species(sub.species)
        c.set_gfunctions(funcs)
        featurise(c, zprec=zprec)
        c.set_network(dims, "tanh", params_now)
        c.set_targets(sub)
        c.set_force_targets(0.1, ds.meta["forces"][:n])
        c.batch_setup(min(args.batch, k))
        c.batch_train_bf16(True)
        g16, _, _ = c.train_gradients("mse")
    out["errors_bf16_vs_fp64"] = {
        "structures": k, "gradient_rel": float(f"{max(float(np.linalg.norm(g16[s] - g64[s]) / np.linalg.norm(g64[s])) for s in range(g64.shape[0])):.3g}")}
    return out


def lbfgs_leg(args):
    """L-BFGS at full history (memory 1000, the reference's default): the optimiser's cost per
    iteration on the C3 networks (three sub-networks of 15,210 parameters) once every one of
    the 1,000 history slots holds a pair, against its cost with 10 slots.  The iterations run
    the full training step on a 64-structure C3 sample, without line search and with the
    quasi-Newton step capped at the maximal displacement, so that every iteration adds a pair;
    the optimiser's launches (gradient preparation, history update, inner products,
    recursion, combination, step) are timed with CUDA events over 20 iterations."""
    from fortnet_gb300 import api, synthetic

    cfg = synthetic.CONFIGS["C3"]
    ds = synthetic.generate(cfg, nstruct=64)
    funcs = synthetic.gfunctions(cfg)
    dims = synthetic.network_dims(cfg)
    params = synthetic.normal_params(dims, len(cfg.atomic_numbers), cfg.seed)
    out = {"memory": 1000, "parameters_per_species": None, "species": len(cfg.atomic_numbers)}
    with api.Context(api.FP32) as c:
        c.upload(ds)
        c.set_species(ds.species)
        c.set_gfunctions(funcs)
        featurise(c, weights=ds.weights)
        c.set_network(dims, "tanh", params)
        c.set_targets(ds)
        out["parameters_per_species"] = int(c.params().shape[1])
        c.optimizer_init("lbfgs", 1e-30, 1e-6, 0.05, memory=1000, linemin=False,
                         qn_max_disp=True)

        def measure(iters=20):
            c.synchronize()
            c.profile(True)
            c.profile_reset()
            for _ in range(iters):
                c.train_iteration("mse")
            c.synchronize()
            ms, n = c.profile_read("optimizer")
            c.profile(False)
            return round(ms / iters, 4)

        for _ in range(10):
            c.train_iteration("mse")
        out["ms_per_iteration_10_slots"] = measure()
        t0 = time.perf_counter()
        filled = 30
        while filled < 1000 + 30 and time.perf_counter() - t0 < 600:
            for _ in range(100):
                c.train_iteration("mse")
            c.synchronize()
            filled += 100
        out["ms_per_iteration_1000_slots"] = measure()
        out["iterations_before_timing"] = filled
        out["slots_written"] = min(1000, filled)
        # the history's FP64 work per iteration at memory m and n parameters per sub-network:
        # the new pair against every slot (S^T y, Y^T y, S^T g, Y^T g: 4 m n FMAs), the
        # combination over S and Y (2 m n) and the m x m matrix-vector products (about 4 m^2),
        # against the device's measured FP64 FMA rate; the time is the increase from 10 to
        # 1,000 slots
        _, _, fp64 = c.probe_peaks()
        n, m, nsp = out["parameters_per_species"], 1000, out["species"]
        dm = m - 10
        flop = 2.0 * nsp * (6.0 * dm * n + 4.0 * (m * m - 100))
        dt = (out["ms_per_iteration_1000_slots"] - out["ms_per_iteration_10_slots"]) / 1e3
        if dt > 0:
            out["history_fp64"] = {"achieved": round(flop / dt / 1e12, 3),
                                   "peak": round(fp64, 3), "unit": "TFLOP/s",
                                   "frac": round(flop / dt / 1e12 / fp64, 3),
                                   "bound": "fp64 (the GPU's FP64 rate is 1/64 of its FP32 "
                                            "rate; the history is kept in FP64)"}
        out["fill_seconds"] = round(time.perf_counter() - t0, 2)
        out["loss"] = float(f"{c.last_losses()[0]:.4g}")
    return out


def serving_leg(args):
    """The C5 serving stream through the public service API (include/fnetg_serve.h): Poisson
    arrivals at 2,000 req/s, each request one three-species periodic structure of 16-4,096
    atoms (log-uniform) drawn from a pool of distinct structures, energies + forces of the
    trained C4 model (66-64-64-1): once with the plain FP32 kernels, once with the network
    passes on the tensor cores (BF16 forward and input Jacobian, FP32 ACSF and forces).
    Latency = completion - scheduled arrival, so a late submission counts against the
    service."""
    from fortnet_gb300 import api, synthetic

    cfg = synthetic.CONFIGS["C5"]
    pool = synthetic.generate(cfg, nstruct=args.serve_pool, targets=False)
    params, zprec, funcs, dims, model_rec = c4_model(args)
    reqs = []
    for s in range(pool.nstruct):
        a, b = pool.atom_offsets[s], pool.atom_offsets[s + 1]
        reqs.append((np.ascontiguousarray(pool.atnum[a:b], dtype=np.int32),
                     np.ascontiguousarray(pool.coords[a:b]), np.ascontiguousarray(pool.latvecs[s])))
    warm, n = args.serve_warmup, args.serve_requests
    arr = synthetic.arrivals(warm + n, seed=cfg.seed)
    pick = np.random.default_rng(cfg.seed + 11).integers(0, len(reqs), size=warm + n)
    import gc
    import queue as _queue

    sys.setswitchinterval(0.0002)  # the submitter spins before each arrival

    def stream(tensor_cores):
        gc.collect()
        gc.disable()  # no collector pauses in the load generator while the stream runs
        pending = _queue.Queue()
        lat = np.zeros(warm + n)
        done_ns = np.zeros(warm + n, dtype=np.int64)
        with api.Server(cfg.atomic_numbers, funcs, zprec, dims, "tanh", params,
                        precision=api.FP32, lanes=args.serve_lanes,
                        tensor_cores=tensor_cores) as srv:
            def waiter():
                for _ in range(warm + n):
                    k, t, na = pending.get()
                    _, _, lat[k] = srv.wait(t, na, timeout=120.0)
                    done_ns[k] = srv.clock_ns()

            th = threading.Thread(target=waiter)
            th.start()
            t0 = srv.clock_ns() + 50_000_000
            for k in range(warm + n):
                target = t0 + int(arr[k] * 1e9)
                while True:
                    dt = target - srv.clock_ns()
                    if dt <= 0:
                        break
                    if dt > 300_000:
                        time.sleep((dt - 200_000) / 1e9)
                an, xyz, lv = reqs[pick[k]]
                t, na = srv.submit(an, xyz, lv, arrival_ns=target)
                pending.put((k, t, na))
            th.join()
            gc.enable()
            st = srv.stats()
        meas = lat[warm:]
        atoms = int(sum(len(reqs[pick[k]][0]) for k in range(warm, warm + n)))
        span = (done_ns[warm:].max() - (t0 + int(arr[warm] * 1e9))) / 1e9
        return {
            "p50_ms": round(float(np.percentile(meas, 50)), 3),
            "p99_ms": round(float(np.percentile(meas, 99)), 3),
            "mean_ms": round(float(np.mean(meas)), 3), "max_ms": round(float(np.max(meas)), 3),
            "atoms_per_s": round(atoms / span, 1),
            "offered_atoms_per_s": round(atoms / (arr[-1] - arr[warm]), 1),
            "lanes": st["lanes"], "batches": st["batches"],
            "mean_batch_requests": round(st["requests"] / max(st["batches"], 1), 2),
            "max_batch_requests": st["max_batch_requests"], "max_in_flight": st["max_in_flight"],
            "max_batch_ms": round(1e3 * st["max_batch_s"], 3),
            "device_bytes": st["device_bytes"]}

    plain = stream(False)
    tc = stream(True)
    # both services against an FP64 run of the plain kernels on the first pool structures;
    # energies relative to sum_i |o_i| of the FP64 atomic outputs
    chk = list(range(min(16, len(reqs))))
    res = {}
    for key, prec, tcores in (("fp32", api.FP32, False), ("bf16", api.FP32, True),
                              ("fp64", api.FP64, False)):
        with api.Server(cfg.atomic_numbers, funcs, zprec, dims, "tanh", params, precision=prec,
                        lanes=1, tensor_cores=tcores) as s2:
            ts = [s2.submit(*reqs[k]) for k in chk]
            res[key] = [s2.wait(t, na, timeout=120.0) for t, na in ts]
    sub = first_structures(pool, len(chk))
    with api.Context(api.FP64) as c:
        c.upload(sub)
        c.set_species(sub.species)
        c.set_gfunctions(funcs)
        c.acsf(download=False)
        c.zscore(zprec=zprec)
        c.set_network(dims, "tanh", params)
        at64, _ = c.predict(atomic=True)
    mag = np.add.reduceat(np.abs(at64[:, 0]), sub.atom_offsets[:-1])

    def errs(key):
        e = max(abs(a[0][0] - b[0][0]) / m for a, b, m in zip(res[key], res["fp64"], mag))
        f = max(float(np.max(np.abs(a[1] - b[1])) / np.max(np.abs(b[1])))
                for a, b in zip(res[key], res["fp64"]))
        return {"structures": len(chk), "energy_rel": float(f"{e:.3g}"),
                "energy_metric": "|E - E64| / sum_i |o_i,64|", "force_rel_of_max": float(f"{f:.3g}")}

    return {
        "workload": f"C5: Poisson {synthetic.C5_RATE:.0f} req/s, 16-4096 atoms log-uniform "
                    f"(pool of {pool.nstruct} structures), model 66-64-64-1 tanh, energies + forces",
        "requests": n, "warmup_requests": warm, "dtype": "f32",
        **plain,
        "fp32_vs_fp64": errs("fp32"),
        "tensor_cores": {"dtype": "bf16 network passes, f32 ACSF and forces", **tc,
                         "vs_fp64": errs("bf16")},
        "model": model_rec,
    }


def first_structures(ds, k):
    """The first k structures of a dataset."""
    from fortnet_gb300.fnetdata import Dataset

    off = ds.atom_offsets[:k + 1]
    n = int(off[-1])
    return Dataset(atom_offsets=off, coords=ds.coords[:n], atnum=ds.atnum[:n],
                   species=ds.species[:n], periodic=ds.periodic[:k], latvecs=ds.latvecs[:k],
                   atomic_numbers=ds.atomic_numbers, weights=ds.weights[:k],
                   atomic_weights=ds.atomic_weights[:n], global_targets=ds.global_targets[:k],
                   atomic_targets=ds.atomic_targets[:n])


def cpu_step(ds, funcs, dims, params, zprec, nthreads):
    """The same step on the oracle (the reference's algorithm restated on the CPU, with the
    reference's loop structure): featurise, one L-BFGS iteration of the full-batch loop
    (gradient, update, gradient at the new parameters), energies of every structure."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    vals = O.acsf(ds, funcs, mode=0, nthreads=nthreads)
    feats = O.zscore_apply(vals, zprec)
    dd, pred = O.train_gradients(dims, "tanh", params, feats, ds)
    g, _ = O.update_prepare(dims, "tanh", params, dd, 0.0, 0.0, float(ds.weights.sum()))
    newp = np.stack([O.Lbfgs(params[s], 1e-20, 1e-6, 1e4, 1000, True, False).next(0.0, g[s])[0]
                     for s in range(params.shape[0])])
    dd, _ = O.train_gradients(dims, "tanh", newp, feats, ds)
    out = O.predict(dims, "tanh", newp, feats, ds.species)
    return np.add.reduceat(out[:, 0], ds.atom_offsets[:-1])


def cpu_sample(args, max_atoms, nstruct):
    """A bounded sample of the workload: the first `nstruct` structures of at most `max_atoms`
    atoms, in dataset order (the oracle's featurisation costs O(atoms^2) per structure)."""
    from fortnet_gb300 import synthetic

    cfg = synthetic.CONFIGS[args.config]
    ds = synthetic.generate(cfg, nstruct=max(8 * nstruct, 64), workers=1)
    n = np.diff(ds.atom_offsets)
    idx = [int(s) for s in np.flatnonzero(n <= max_atoms)][:nstruct]
    from fortnet_gb300.fnetdata import Dataset

    off = ds.atom_offsets
    rows = np.concatenate([np.arange(off[s], off[s + 1]) for s in idx])
    noff = np.concatenate([[0], np.cumsum([off[s + 1] - off[s] for s in idx])]).astype(np.int64)
    sub = Dataset(atom_offsets=noff, coords=np.ascontiguousarray(ds.coords[rows]),
                  atnum=ds.atnum[rows], species=ds.species[rows], periodic=ds.periodic[idx],
                  latvecs=np.ascontiguousarray(ds.latvecs[idx]), atomic_numbers=ds.atomic_numbers,
                  weights=ds.weights[idx], atomic_weights=ds.atomic_weights[rows],
                  global_targets=np.ascontiguousarray(ds.global_targets[idx]),
                  atomic_targets=ds.atomic_targets[rows])
    return cfg, sub


def cpu_baseline(args, threads):
    from fortnet_gb300 import synthetic

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    cfg, ds = cpu_sample(args, args.cpu_max_atoms, args.cpu_sample)
    funcs = synthetic.gfunctions(cfg)
    dims = synthetic.network_dims(cfg)
    params = O.Ranlux(cfg.seed).init_bpnn(dims, "tanh", len(cfg.atomic_numbers))
    zprec = O.zscore_stats(O.acsf(ds, funcs, mode=1), ds)
    t0 = time.perf_counter()
    cpu_step(ds, funcs, dims, params, zprec, threads)
    dt = time.perf_counter() - t0
    return {"value": round(ds.ntot / dt, 2), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{ds.nstruct} {args.config} structures of <= {args.cpu_max_atoms} atoms "
                      f"({ds.ntot} atoms), one step: featurise + one L-BFGS iteration + energies; "
                      f"the oracle restates the reference loop structure (per-(atom, G) "
                      f"neighbour rebuild, per-atom network evaluation)", "seconds": round(dt, 2)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # only the oracle's library is loaded on this arm (the synthetic generator is numpy)
    from fortnet_gb300 import synthetic

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    cfg, ds = cpu_sample(args, args.cpu_max_atoms, args.ref_sample)
    funcs = synthetic.gfunctions(cfg)
    dims = synthetic.network_dims(cfg)
    params = O.Ranlux(cfg.seed).init_bpnn(dims, "tanh", len(cfg.atomic_numbers))
    zprec = O.zscore_stats(O.acsf(ds, funcs, mode=1, nthreads=threads), ds)
    for _ in range(min(args.warmup, 1)):
        cpu_step(ds, funcs, dims, params, zprec, threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cpu_step(ds, funcs, dims, params, zprec, threads)
        times.append(time.perf_counter() - t0)
    dt = float(np.mean(times))
    v = ds.ntot / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(v, 2), "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic (seeded {args.config} generator)",
        "config": {"workload": f"{args.config} sample: {ds.nstruct} structures of <= "
                               f"{args.cpu_max_atoms} atoms, {ds.ntot} atoms; featurise + one "
                               f"L-BFGS iteration + energies"},
        "cpu_baseline": {"value": round(v, 2), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{ds.nstruct} {args.config} structures per step (oracle "
                                   f"restatement of the reference algorithm; the Fortran program "
                                   f"cannot be built here)"},
        "e2e": {"value": round(v, 2), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="C3")
    ap.add_argument("--nstruct", type=int, default=None)
    ap.add_argument("--batch", type=int, default=BATCH, help="structures per mini-batch")
    ap.add_argument("--lr", type=float, default=1e-6,
                    help="learning rate of the mini-batch steepest descent")
    ap.add_argument("--plain-steps", type=int, default=5)
    ap.add_argument("--cpu-sample", type=int, default=4)
    ap.add_argument("--cpu-max-atoms", type=int, default=128)
    ap.add_argument("--ref-sample", type=int, default=12)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--acc-epochs", type=int, default=60,
                    help="batched-form epochs of the test-set accuracy comparison (0: skip)")
    ap.add_argument("--acc-lrs", type=float, nargs="+", default=[1e-5, 1e-4, 1e-3, 1e-2])
    ap.add_argument("--acc-test-structs", type=int, default=400)
    ap.add_argument("--no-lbfgs", action="store_true",
                    help="skip the L-BFGS full-history measurement")
    ap.add_argument("--serve-requests", type=int, default=20000,
                    help="requests of the C5 serving stream (0: skip the serving leg)")
    ap.add_argument("--serve-warmup", type=int, default=1000)
    ap.add_argument("--serve-pool", type=int, default=64)
    ap.add_argument("--serve-lanes", type=int, default=3)
    ap.add_argument("--model-structs", type=int, default=96,
                    help="C4 structures the served model is trained on")
    ap.add_argument("--model-iters", type=int, default=600)
    ap.add_argument("--c4-structs", type=int, default=5000)
    ap.add_argument("--c4-iters", type=int, default=3,
                    help="timed force-loss training iterations on C4 (0: skip the leg)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

#!/usr/bin/env python
"""Benchmark: boosting iterations per second of the GB300 tree learner.

Workload: L2 regression, 10,000,000 rows x 100 float32 features (70 N(0,1), 30 integer 0..15,
10% NaN), target = sum of 20 random step functions + N(0, 0.1); max_bin 255, num_leaves 255,
learning rate 0.1. Synthetic data of that shape (seeded) stands in for real data.

A step is one boosting iteration: L2 gradients on the device, one tree (histograms, split
search, partition, bookkeeping), and the score update. Two forms of the learner are timed:
  * quantized+batched: int8 discretized gradients, exact integer histograms, and the whole
    grow loop of an iteration replayed as one CUDA graph  -> the reported `value`;
  * plain: fp32 compensated histograms with f64 gains and one host round trip per split.

`e2e` is the same metric through the C ABI with host buffers: every step copies that step's
gradients / hessians from pinned host memory to the device inside the timed region and reads
the training loss back.

`--impl reference` times the CPU learner (the oracle port of the reference's tree learner, with
all host threads) on the same workload: all rows, the quantized config of `value`, every step a
full boosting iteration; its rows are binned by the oracle's own restatement of the bin mappers.

Multi-GPU (`--gpus N`, torchrun): independent replicas, one per GPU (the learner adds no
cross-GPU exchange step); value = iterations of all ranks / max time over ranks.
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
K_ZERO_THRESHOLD = float(np.float32(1e-35))
sys.path.insert(0, os.path.join(ROOT, "bankai-lightgbm_gb300"))

METRIC = "iters/s (10M x 100, 255 leaves) quantized+batched vs plain GPU; hist HBM GB/s"
WORKLOAD = ("L2 regression 10M x 100 (70 N(0,1) + 30 int 0..15, 10% NaN), max_bin 255, 255 leaves, "
            "lr 0.1; step = device gradients + 1 tree + score update")


# DRAM bytes (read + write) per algorithmic byte of the quantized histogram kernel, from one ncu
# capture of every k_hist_int launch of one 255-leaf tree on this workload at 2M rows (the bins,
# 2M x 128 bytes, are larger than L2; the capture's metrics take one pass):
#   python bench.py --hist-traffic --rows 2000000 &&
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum --clock-control none \
#       -k regex:k_hist_int --csv --log-file ht2m.csv python bench.py --hist-traffic --rows 2000000
# 1.148 GB read + 3.1 MB written for 0.841 GB of algorithmic bytes over the 254 launches.
HIST_TRAFFIC_PER_BYTE = (1.148e9 + 3.1e6) / 0.841278208e9


def _peaks():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 6:
                self.samples.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[2 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def build_dataset(rows, seed=0, heldout=False, device_binning=False):
    """Training rows, plus (heldout=True) a 20% held-out split from the same generator, binned
    with the training bin mappers. device_binning=True also bins the training rows on the device
    (BinnedDataset.from_dense_device) and returns its timings and whether its bins equal the
    host's."""
    from lgbm_gb300 import BinnedDataset, synthetic
    total = rows + (rows // 4 if heldout else 0)
    X, y = synthetic.l2_steps(n=total, seed=seed)
    threads = min(32, os.cpu_count() or 8)
    t0 = time.time()
    ds = BinnedDataset.from_dense(X[:rows], max_bin=255, min_data_in_leaf=20, threads=threads)
    host_s = time.time() - t0
    binning = _device_binning(X[:rows], ds, threads, host_s) if device_binning else None
    ho = (ds.bin_like(X[rows:], threads=threads), y[rows:]) if heldout else None
    del X
    if device_binning:
        return ds, y[:rows], ho, binning
    return ds, y[:rows], ho


def _device_binning(X, ds, threads, host_s):
    """Device bin construction of the same rows: the whole from_dense_device (host bin mappers
    from the row sample + device binning) and the device binning call alone (CUDA events, median
    of 3), against the host's from_dense time; value bytes read + stored bytes written per second."""
    import torch
    from lgbm_gb300 import BinnedDataset
    Xd = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    torch.cuda.synchronize()
    t0 = time.time()
    dev = BinnedDataset.from_dense_device(Xd, max_bin=255, min_data_in_leaf=20, threads=threads)
    torch.cuda.synchronize()
    full_s = time.time() - t0
    match = bool(np.array_equal(dev.bins.cpu().numpy(), ds.bins))
    times = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = dev.bin_like_device(Xd)
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
        del out
    ms = float(np.median(times))
    n, ncol = Xd.shape
    nbytes = n * ncol * Xd.element_size() + n * dev.num_features
    del Xd, dev
    torch.cuda.empty_cache()
    return {"host_from_dense_s": round(host_s, 2), "device_from_dense_s": round(full_s, 2),
            "device_bin_ms": round(ms, 3), "device_bin_gbs": round(nbytes / (ms * 1e6), 1), "bins_equal": match,
            "values": "f32 [%d x %d] row-major" % (n, ncol)}


def make_cfg(quant, num_leaves=255):
    from lgbm_gb300 import LearnerConfig
    return LearnerConfig(num_leaves=num_leaves, min_data_in_leaf=20, use_quantized_grad=int(quant),
                         num_grad_quant_bins=4, stochastic_rounding=1, seed=0, num_threads=16, fused_madd=1,
                         is_constant_hessian=1)


def run_gpu(args, rank, world):
    import torch
    from lgbm_gb300 import GpuTreeLearner, _lib
    from lgbm_gb300.tree import Tree
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    lr = 0.1
    t0 = time.time()
    ds, y, (ho_bins_np, ho_y), binning = build_dataset(args.rows, heldout=True, device_binning=True)
    prep_s = time.time() - t0
    n = ds.num_data
    label = torch.from_numpy(y).cuda()
    ho_bins = torch.from_numpy(ho_bins_np).cuda()
    ho_label = torch.from_numpy(ho_y.astype(np.float64)).cuda()
    m_ho = ho_bins.shape[1]
    peak, peak_kind = _peaks()

    shapes = {}

    def form(quant, loop_mode, steps, warmup, e2e=False, timing=False):
        learner = GpuTreeLearner(ds, make_cfg(quant, args.leaves), loop_mode=loop_mode)
        learner.set_timing(timing)
        stream = torch.cuda.ExternalStream(learner.stream())
        score = torch.full((n,), float(y.astype(np.float64).mean()), dtype=torch.float64, device="cuda")
        gbuf, hbuf = learner.gradient_buffers()
        torch.cuda.synchronize()  # score and labels are written on torch's stream
        if args.autotune:
            # launch shape from trial trees on the first iteration's gradients (cached per shape
            # class, so only the first learner of each form kind pays for the trials)
            learner.objective_gradients(0, score.data_ptr(), label.data_ptr())
            learner.autotune(gbuf, hbuf, on_device=True, trials=2)
        shapes[(quant, loop_mode)] = learner.launch_shape()
        pin_g = torch.empty(n, dtype=torch.float32).pin_memory() if e2e else None
        pin_h = torch.empty(n, dtype=torch.float32).pin_memory() if e2e else None
        stats = dict(hist_ms=0.0, hist_bytes=0.0, train_ms=0.0, search_ms=0.0, part_ms=0.0, leaves=0, loss=None,
                     launches=[])
        total_ms = 0.0
        trees = []

        def step(timed):
            nonlocal total_ms
            if e2e:
                # this step's inputs live in pinned host memory (computed by the objective from the
                # current score outside the timed region)
                learner.objective_gradients(0, score.data_ptr(), label.data_ptr())
                torch.cuda.synchronize()
                pin_g.copy_(_device_view(gbuf, n))
                pin_h.copy_(_device_view(hbuf, n))
                torch.cuda.synchronize()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            if e2e:
                splits, lv, roots, nls = _host_train(learner, pin_g, pin_h)
            else:
                learner.objective_gradients(0, score.data_ptr(), label.data_ptr())
                splits, lv, roots, nls = learner.train_raw(gbuf, hbuf, on_device=True)
            # Tree::apply_shrinkage on the leaf values (tree.rs:446-463); the tree object itself is
            # assembled after the timed region
            vals = lv[0] * lr
            vals[np.abs(vals) <= K_ZERO_THRESHOLD] = 0.0
            learner.add_prediction_to_score(vals, score.data_ptr(), on_device=True)
            trees.append((splits[0, :nls[0] - 1].copy(), lv[0, :nls[0]].copy(), float(roots[0])))
            if e2e:
                stats["loss"] = learner.objective_loss(0, score.data_ptr(), label.data_ptr())
            ev1.record(stream)
            ev1.synchronize()
            if timed:
                total_ms += ev0.elapsed_time(ev1)
                tm = learner.last_timing()
                stats["hist_ms"] += tm["hist_ms"]
                stats["hist_bytes"] += tm["hist_bytes"]
                stats["train_ms"] += tm["total_ms"]
                stats["search_ms"] += tm["search_ms"]
                stats["part_ms"] += tm["partition_ms"]
                stats["leaves"] += int(nls[0])
                if timing:
                    # per histogram launch: (rows of the leaf it builds, its CUDA-event ms)
                    st = learner.last_step_timing()
                    rows = _hist_launch_rows(splits[0, :nls[0] - 1], n, args.leaves)
                    stats["launches"] += [(r, float(t)) for r, t in zip(rows, st[:, 0]) if t >= 0]

        for _ in range(warmup):
            step(False)
        torch.cuda.synchronize()
        for _ in range(steps):
            step(True)
        torch.cuda.synchronize()
        stats["ms_per_step"] = total_ms / max(steps, 1)
        stats["train_ms_per_step"] = stats["train_ms"] / max(steps, 1)
        stats["hist_ms_per_step"] = stats["hist_ms"] / max(steps, 1)
        stats["loss_final"] = learner.objective_loss(0, score.data_ptr(), label.data_ptr())
        # held-out L2 after the same number of trees (outside the timed region)
        ho_score = torch.full((m_ho,), float(y.astype(np.float64).mean()), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for sp, lvals, root in trees:
            t = Tree.from_records(args.leaves, sp, lvals, root, ds.features)
            t.apply_shrinkage(lr)
            learner.predict_add(t, ho_bins.data_ptr(), m_ho, ho_score.data_ptr())
        stats["heldout_l2"] = _l2(ho_score, ho_label)
        stats["iterations"] = len(trees)
        learner.close()
        return stats

    def _host_train(learner, pg, ph):
        """bk_learner_train on host (pinned) gradient buffers: the copy to the device is inside."""
        K, Lv = learner.num_jobs, learner.num_leaves
        from lgbm_gb300.tree import SPLIT_DTYPE
        splits = np.zeros((K, Lv - 1), dtype=SPLIT_DTYPE)
        lv = np.zeros((K, Lv))
        roots = np.zeros(K)
        nls = np.zeros(K, np.int32)
        _lib.check(learner.lib.bk_learner_train(learner.h, pg.data_ptr(), ph.data_ptr(), 0, None, 0,
                                                splits.ctypes.data, lv.ctypes.data, roots.ctypes.data,
                                                nls.ctypes.data), "bk_learner_train")
        return splits, lv, roots, nls

    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    main = form(True, 1, args.steps, args.warmup)
    clk = clocks.stop()
    # the histogram launches timed one by one with CUDA events (event nodes in the graph), in a
    # separate run so that they do not perturb the headline number
    roof = form(True, 1, args.steps, 1, timing=True)
    plain = form(False, 0, args.steps, args.warmup)
    # the float learner in the same graph form as `value`: the quantization gain on its own
    float_graph = form(False, 1, args.steps, args.warmup)
    e2e = form(True, 1, args.steps, 1, e2e=True)
    multiclass = _side(run_multiclass, args) if args.multiclass_rows > 0 else None
    batched_jobs = _side(run_batched_jobs, args) if args.batch_jobs > 0 else None
    binary = _side(run_binary, args) if args.binary_rows > 0 else None
    ms, value = aggregate_ranks(main["ms_per_step"], world)
    hist_gbs = roof["hist_bytes"] / (roof["hist_ms"] * 1e6) if roof["hist_ms"] > 0 else None
    hist_launches = (args.leaves - 1) * args.steps  # one histogram launch per split step of a tree
    # per step: objective gradients, row init, discretization (4), root sums (2), tree begin, three
    # kernels per split (histogram, search, partition), the last split's bookkeeping, score update
    launches_per_step = 1 + 1 + 4 + 2 + 1 + 3 * (args.leaves - 1) + 1 + 1
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "iters/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int8 grad/hess, int64 histograms, f64 gains", "data": "synthetic (seeded)",
        "config": _config(ds, args, world),
        "forms": {"quantized_graph": {"iters_per_s": round(1000.0 / main["ms_per_step"], 4),
                                      "train_call_ms": round(main["train_ms_per_step"], 3),
                                      "hist_ms": round(roof["hist_ms_per_step"], 3),
                                      "search_ms": round(roof["search_ms"] / max(args.steps, 1), 3),
                                      "partition_ms": round(roof["part_ms"] / max(args.steps, 1), 3),
                                      "train_l2": main["loss_final"], "heldout_l2": main["heldout_l2"],
                                      "iterations": main["iterations"],
                                      "launch_shape": _shape_dict(shapes.get((True, 1)), args.autotune)},
                  "plain_float_stepwise": {"iters_per_s": round(1000.0 / plain["ms_per_step"], 4),
                                           "train_l2": plain["loss_final"], "heldout_l2": plain["heldout_l2"],
                                           "iterations": plain["iterations"],
                                           "launch_shape": _shape_dict(shapes.get((False, 0)), args.autotune)},
                  "float_graph": {"iters_per_s": round(1000.0 / float_graph["ms_per_step"], 4),
                                  "train_l2": float_graph["loss_final"], "heldout_l2": float_graph["heldout_l2"],
                                  "iterations": float_graph["iterations"],
                                  "launch_shape": _shape_dict(shapes.get((False, 1)), args.autotune)},
                  "heldout_l2_delta": main["heldout_l2"] - plain["heldout_l2"], "heldout_rows": m_ho,
                  "multiclass_k10": multiclass, "batched_jobs": batched_jobs, "binary_quantized_200": binary},
        "e2e": {"value": round(world * 1000.0 / e2e["ms_per_step"], 4), "unit": "iters/s",
                "h2d_bytes_per_step": 2 * 4 * ds.num_data,
                "d2h_bytes_per_step": 112 * (args.leaves - 1) + 8 * args.leaves + 8 + 8},
        "roofline": {"bound": "hbm", "achieved": round(hist_gbs, 1) if hist_gbs else None, "peak": peak,
                     "unit": "GB/s", "frac": round(hist_gbs / peak, 4) if hist_gbs else None,
                     "traffic": round(HIST_TRAFFIC_PER_BYTE * roof["hist_bytes"] / hist_launches, 0),
                     "algorithmic_bytes_per_launch": round(roof["hist_bytes"] / hist_launches, 0),
                     "traffic_source": "ncu capture of one tree's 254 launches at 2M rows (DRAM bytes per "
                                       "algorithmic byte, %.3f) x this run's algorithmic bytes per launch"
                                       % HIST_TRAFFIC_PER_BYTE,
                     "kernel": "k_hist_int (quantized histogram)", "peak_kind": peak_kind,
                     "by_leaf_size": _roofline_by_leaf_size(roof["launches"], ds, n, peak)},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clk,
        "prep_s": round(prep_s, 1),
        "binning": binning,
    }
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(ds, y, leaves=args.leaves)
    line["summary"] = _summary(line)
    return line


def _summary(line):
    """The line's key figures once more, compactly, at its end (a log that keeps only the tail of
    the output still shows them)."""
    f = line["forms"]

    def get(d, *keys):
        for k in keys:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d
    return {"iters_per_s": {"quantized_graph": line["value"], "float_graph": get(f, "float_graph", "iters_per_s"),
                            "plain_float_stepwise": get(f, "plain_float_stepwise", "iters_per_s"),
                            "e2e": line["e2e"]["value"], "cpu_oracle": get(line, "cpu_baseline", "value")},
            "heldout_l2": {"quantized": get(f, "quantized_graph", "heldout_l2"),
                           "float_graph": get(f, "float_graph", "heldout_l2"),
                           "delta_vs_float": f.get("heldout_l2_delta")},
            "multiclass_k10_iters_per_s": [get(f, "multiclass_k10", "quantized_graph", "iters_per_s"),
                                           get(f, "multiclass_k10", "plain_float_stepwise", "iters_per_s")],
            "binary_200_iters_per_s": [get(f, "binary_quantized_200", "quantized_graph", "iters_per_s"),
                                       get(f, "binary_quantized_200", "plain_float_stepwise", "iters_per_s")],
            "binary_200_heldout_auc_delta": get(f, "binary_quantized_200", "heldout_auc_delta"),
            "batched_job_iters_per_s": [get(f, "batched_jobs", "group_graph", "job_iters_per_s"),
                                        get(f, "batched_jobs", "batched", "job_iters_per_s"),
                                        get(f, "batched_jobs", "one_by_one", "job_iters_per_s")],
            "hist_roofline_frac": line["roofline"]["frac"]}


def run_multiclass(args):
    """Multiclass softmax, K=10 class trees per iteration grown in one call (each grow-loop kernel
    launched for groups of class trees): 2M x 64 Gaussian-mixture rows (10 components, means
    spread 2.0), max_bin 63, 63 leaves. Quantized + graph form against the plain float form with
    one host round trip per split; iterations per second, training and held-out (20%) multi-class
    log loss."""
    import torch
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig, synthetic
    from lgbm_gb300.tree import Tree
    K, leaves, lr = 10, 63, 0.1
    rows = args.multiclass_rows
    X, y = synthetic.gaussian_mixture(n=rows + rows // 4, F=64, K=K, seed=0)
    threads = min(32, os.cpu_count() or 8)
    ds = BinnedDataset.from_dense(X[:rows], max_bin=63, min_data_in_leaf=20, threads=threads)
    ho_bins = torch.from_numpy(ds.bin_like(X[rows:], threads=threads)).cuda()
    del X
    n, m = ds.num_data, ho_bins.shape[1]
    label = torch.from_numpy(y[:rows]).cuda()
    ho_y = torch.from_numpy(y[rows:].astype(np.int64)).cuda()
    prior = np.bincount(y[:rows].astype(np.int64), minlength=K) / float(rows)
    init = torch.tensor(np.log(np.maximum(prior, 1e-15)), dtype=torch.float64, device="cuda")[:, None]

    def form(quant, loop_mode, steps, warmup):
        cfg = LearnerConfig(num_leaves=leaves, min_data_in_leaf=20, use_quantized_grad=int(quant),
                            num_grad_quant_bins=4, stochastic_rounding=1, seed=0, num_threads=16, fused_madd=1)
        learner = GpuTreeLearner(ds, cfg, num_jobs=K, loop_mode=loop_mode)
        stream = torch.cuda.ExternalStream(learner.stream())
        score = (init.expand(K, n)).contiguous()
        gbuf, hbuf = learner.gradient_buffers()
        torch.cuda.synchronize()
        if args.autotune:
            learner.objective_gradients(2, score.data_ptr(), label.data_ptr())
            learner.autotune(gbuf, hbuf, on_device=True, trials=2)
        shape = learner.launch_shape()
        trees, total_ms = [], 0.0
        for it in range(warmup + steps):
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            learner.objective_gradients(2, score.data_ptr(), label.data_ptr())
            splits, lv, roots, nls = learner.train_raw(gbuf, hbuf, on_device=True)
            vals = lv * lr
            vals[np.abs(vals) <= K_ZERO_THRESHOLD] = 0.0
            learner.add_prediction_to_score(vals, score.data_ptr(), on_device=True)
            ev1.record(stream)
            ev1.synchronize()
            if it >= warmup:
                total_ms += ev0.elapsed_time(ev1)
            trees.append([(splits[k, :nls[k] - 1].copy(), lv[k, :nls[k]].copy(), float(roots[k])) for k in range(K)])
        train_loss = learner.objective_loss(2, score.data_ptr(), label.data_ptr())
        ho = (init.expand(K, m)).contiguous()
        torch.cuda.synchronize()
        for per_class in trees:
            for k, (sp, lvals, root) in enumerate(per_class):
                t = Tree.from_records(leaves, sp, lvals, root, ds.features)
                t.apply_shrinkage(lr)
                learner.predict_add(t, ho_bins.data_ptr(), m, ho[k].data_ptr())
        torch.cuda.synchronize()
        ho_loss = _multi_logloss(ho, ho_y)
        learner.close()
        return {"iters_per_s": round(1000.0 * steps / total_ms, 3), "ms_per_iter": round(total_ms / steps, 3),
                "train_logloss": round(train_loss, 6), "heldout_logloss": round(ho_loss, 6),
                "iterations": len(trees), "launch_shape": _shape_dict(shape, args.autotune)}

    q = form(True, 1, args.steps, args.warmup)
    p = form(False, 0, args.steps, args.warmup)
    return {"workload": "multiclass softmax K=10, %d x 64 Gaussian mixture, max_bin 63, 63 leaves; step = device "
                        "gradients + 10 class trees in one call + score update" % n,
            "quantized_graph": q, "plain_float_stepwise": p,
            "heldout_logloss_delta": round(q["heldout_logloss"] - p["heldout_logloss"], 6)}


def run_batched_jobs(args):
    """Independent binary-classification jobs: rows log-uniform in [5,000, 500,000], features
    uniform in [20, 300] (N(0,1), 1% NaN), logistic labels from per-job random linear models,
    max_bin drawn from {15, 63, 255}, 31 leaves, quantized gradients. Every job has its own
    learner, dataset and stream. One iteration = device binary gradients + one tree + device score
    update for every job; timed three ways: the jobs one after another (bk_learner_train per job),
    all jobs in one bk_learners_train_batch call per iteration (one stream per job), and all jobs
    as one CUDA graph per iteration (bk_learner_group_train) with the launch policy the group's
    autotuner picks (bk_learner_group_autotune). Host wall clock around each iteration loop,
    bracketed by device synchronization (the work spans many streams)."""
    import torch
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig, LearnerGroup, synthetic, train_batch
    threads = min(32, os.cpu_count() or 8)
    jobs = []
    t0 = time.time()
    for X, y, mb in synthetic.batched_jobs(args.batch_jobs, seed=7):
        ds = BinnedDataset.from_dense(X, max_bin=mb, min_data_in_leaf=20, threads=threads)
        jobs.append((ds, torch.from_numpy(y).cuda(), mb))
        del X
    prep_s = time.time() - t0
    rows = [ds.num_data for ds, _, _ in jobs]
    feats = [ds.num_features for ds, _, _ in jobs]

    def make():
        out = []
        for i, (ds, label, mb) in enumerate(jobs):
            cfg = LearnerConfig(num_leaves=31, min_data_in_leaf=20, use_quantized_grad=1, num_grad_quant_bins=4,
                                stochastic_rounding=1, seed=i, num_threads=16, fused_madd=1)
            L = GpuTreeLearner(ds, cfg)
            score = torch.zeros(ds.num_data, dtype=torch.float64, device="cuda")
            gb, hb = L.gradient_buffers()
            if args.autotune:
                torch.cuda.synchronize()
                L.objective_gradients(1, score.data_ptr(), label.data_ptr())
                L.autotune(gb, hb, on_device=True, trials=1)
            out.append((L, score, label, (gb, hb)))
        torch.cuda.synchronize()
        return out

    def run(learners, batched, iters, group=None):
        for L, score, label, _ in learners:
            score.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(iters):
            if group is not None:
                for L, score, label, _ in learners:
                    L.objective_gradients(1, score.data_ptr(), label.data_ptr())
                group.train([x[3][0] for x in learners], [x[3][1] for x in learners], shrinkage=0.1,
                            scores=[x[1].data_ptr() for x in learners])
            elif batched:
                for L, score, label, _ in learners:
                    L.objective_gradients(1, score.data_ptr(), label.data_ptr())
                train_batch([x[0] for x in learners], [x[3][0] for x in learners], [x[3][1] for x in learners],
                            on_device=True, shrinkage=0.1, scores=[x[1].data_ptr() for x in learners])
            else:
                for L, score, label, (gb, hb) in learners:
                    L.objective_gradients(1, score.data_ptr(), label.data_ptr())
                    _, lv, _, nls = L.train_raw(gb, hb, on_device=True)
                    if nls[0] > 1:
                        vals = lv * 0.1
                        vals[np.abs(vals) <= K_ZERO_THRESHOLD] = 0.0
                        L.add_prediction_to_score(vals, score.data_ptr(), on_device=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        loss = float(np.mean([L.objective_loss(1, score.data_ptr(), label.data_ptr()) for L, score, label, _ in learners]))
        return dt, loss

    t0 = time.time()
    learners = make()
    setup_s = time.time() - t0
    run(learners, True, 1)  # warm-up: graph capture of every learner
    run(learners, False, 1)
    seq_s, seq_loss = run(learners, False, args.batch_iters)
    bat_s, bat_loss = run(learners, True, args.batch_iters)
    # one CUDA graph per iteration for all jobs, with the group's autotuned launch policy
    group = LearnerGroup([x[0] for x in learners])
    t0 = time.time()
    for L, score, label, _ in learners:
        score.zero_()
        L.objective_gradients(1, score.data_ptr(), label.data_ptr())
    torch.cuda.synchronize()
    policy = group.autotune([x[3][0] for x in learners], [x[3][1] for x in learners], trials=2)
    tune_s = time.time() - t0
    run(learners, True, 1, group)  # warm-up: the group graph's capture
    grp_s, grp_loss = run(learners, True, args.batch_iters, group)
    group.close()
    for L, _, _, _ in learners:
        L.close()
    J, it = len(jobs), args.batch_iters
    return {"workload": "%d independent binary jobs, rows log-uniform 5k-500k (total %d), features 20-300 (mean %.0f), "
                        "max_bin in {15, 63, 255}, 31 leaves, quantized; %d iterations each"
                        % (J, sum(rows), float(np.mean(feats)), it),
            "one_by_one": {"job_iters_per_s": round(J * it / seq_s, 2), "s": round(seq_s, 3),
                           "mean_train_logloss": round(seq_loss, 6)},
            "batched": {"job_iters_per_s": round(J * it / bat_s, 2), "s": round(bat_s, 3),
                        "mean_train_logloss": round(bat_loss, 6)},
            "group_graph": {"job_iters_per_s": round(J * it / grp_s, 2), "s": round(grp_s, 3),
                            "mean_train_logloss": round(grp_loss, 6),
                            "policy": {"launch_overlap": policy[0], "hist_min_rows_per_cta": policy[1],
                                       "hist_ctas_per_job": policy[2], "partition_ctas": policy[3]},
                            "autotune_s": round(tune_s, 2)},
            "speedup": round(seq_s / bat_s, 3), "speedup_group": round(seq_s / grp_s, 3), "prep_s": round(prep_s, 1),
            "learner_setup_s": round(setup_s, 2), "autotuned": bool(args.autotune)}


def _l2(score, label):
    """Mean squared error (metric/regression.rs `l2`)."""
    return float(((score - label.to(score.dtype)) ** 2).mean().item())


def _multi_logloss(score, label):
    """Mean multi-class log loss of raw scores [K, n] (metric/multiclass.rs `multi_logloss`:
    -log of the softmax probability of the label class)."""
    import torch
    return float((torch.logsumexp(score, 0) - score.gather(0, label.long()[None, :])[0]).mean().item())


def _auc(score, label):
    """Area under the ROC curve with average ranks for tied scores (metric/binary.rs AUC)."""
    import torch
    order = torch.argsort(score)
    s = score[order]
    y = label[order].double()
    _, inverse, counts = torch.unique_consecutive(s, return_inverse=True, return_counts=True)
    ends = torch.cumsum(counts, 0).double()
    avg_rank = ends - (counts.double() - 1.0) / 2.0  # 1-based average rank of each tie group
    ranks = avg_rank[inverse]
    pos = float(y.sum().item())
    neg = float(len(y)) - pos
    return float(((ranks * y).sum().item() - pos * (pos + 1.0) / 2.0) / (pos * neg))


def run_binary(args):
    """Binary classification with quantized gradients: rows x 200 float32 features (100 N(0,1) and
    100 uniform(-1, 1), 5% NaN), labels from a logistic model on a random sparse linear term
    (20 nonzero weights), 255 leaves; the quantized form (4 gradient bins, stochastic rounding,
    graph) against the plain float form (one host round trip per split). The values are generated
    on the device (seeded) and binned there (host bin mappers from the row sample); iterations/s
    and the AUC of a 20% held-out split from the same generator."""
    import torch
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig
    from lgbm_gb300.tree import Tree
    rows, F, leaves, lr = args.binary_rows, 200, 255, 0.1
    n_all = rows + rows // 4
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    X = torch.empty((n_all, F), dtype=torch.float32, device="cuda")
    X[:, :F // 2].normal_(generator=gen)
    X[:, F // 2:].uniform_(-1.0, 1.0, generator=gen)
    w = torch.zeros(F, dtype=torch.float32, device="cuda")
    nz = torch.randperm(F, generator=gen, device="cuda")[:F // 10]
    w[nz] = torch.randn(F // 10, generator=gen, device="cuda")
    y = (torch.rand(n_all, generator=gen, device="cuda") < torch.sigmoid(X @ w)).float()
    for c0 in range(0, F, 25):  # NaNs in column blocks (bounded temporary memory)
        blk = X[:, c0:c0 + 25]
        blk[torch.rand(blk.shape, generator=gen, device="cuda") < 0.05] = float("nan")
    torch.cuda.synchronize()
    threads = min(32, os.cpu_count() or 8)
    t0 = time.time()
    ds = BinnedDataset.from_dense_device(X[:rows], max_bin=255, min_data_in_leaf=20, threads=threads)
    ho_bins = ds.bin_like_device(X[rows:])
    torch.cuda.synchronize()
    prep_s = time.time() - t0
    del X
    torch.cuda.empty_cache()
    n, m = ds.num_data, ho_bins.shape[1]
    label, ho_y = y[:rows].contiguous(), y[rows:].contiguous()
    pavg = min(max(float(label.mean().item()), 1e-15), 1.0 - 1e-15)
    init = float(np.log(pavg / (1.0 - pavg)))

    def form(quant, loop_mode, steps, warmup):
        cfg = LearnerConfig(num_leaves=leaves, min_data_in_leaf=20, use_quantized_grad=int(quant),
                            num_grad_quant_bins=4, stochastic_rounding=1, seed=0, num_threads=16, fused_madd=1)
        learner = GpuTreeLearner(ds, cfg, loop_mode=loop_mode)
        stream = torch.cuda.ExternalStream(learner.stream())
        score = torch.full((n,), init, dtype=torch.float64, device="cuda")
        gbuf, hbuf = learner.gradient_buffers()
        torch.cuda.synchronize()
        if args.autotune:
            learner.objective_gradients(1, score.data_ptr(), label.data_ptr())
            learner.autotune(gbuf, hbuf, on_device=True, trials=2)
        trees, total_ms = [], 0.0
        for it in range(warmup + steps):
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            learner.objective_gradients(1, score.data_ptr(), label.data_ptr())
            splits, lv, roots, nls = learner.train_raw(gbuf, hbuf, on_device=True)
            vals = lv * lr
            vals[np.abs(vals) <= K_ZERO_THRESHOLD] = 0.0
            learner.add_prediction_to_score(vals, score.data_ptr(), on_device=True)
            ev1.record(stream)
            ev1.synchronize()
            if it >= warmup:
                total_ms += ev0.elapsed_time(ev1)
            trees.append((splits[0, :nls[0] - 1].copy(), lv[0, :nls[0]].copy(), float(roots[0])))
        train_loss = learner.objective_loss(1, score.data_ptr(), label.data_ptr())
        ho = torch.full((m,), init, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for sp, lvals, root in trees:
            t = Tree.from_records(leaves, sp, lvals, root, ds.features)
            t.apply_shrinkage(lr)
            learner.predict_add(t, ho_bins.data_ptr(), m, ho.data_ptr())
        torch.cuda.synchronize()
        out = {"iters_per_s": round(1000.0 * steps / total_ms, 3), "ms_per_iter": round(total_ms / steps, 3),
               "train_logloss": round(train_loss, 6), "heldout_auc": round(_auc(ho, ho_y), 6),
               "iterations": len(trees), "launch_shape": _shape_dict(learner.launch_shape(), args.autotune)}
        learner.close()
        return out

    q = form(True, 1, args.steps, args.warmup)
    p = form(False, 0, args.steps, args.warmup)
    return {"workload": "binary, %d x %d (N(0,1) / uniform halves, 5%% NaN), sparse logistic labels, 255 leaves; "
                        "step = device gradients + 1 tree + score update" % (n, ds.num_features),
            "quantized_graph": q, "plain_float_stepwise": p,
            "heldout_auc_delta": round(q["heldout_auc"] - p["heldout_auc"], 6), "prep_s": round(prep_s, 1)}


def _side(fn, args):
    """A side form's result, or its error (a side form never takes the headline line down)."""
    try:
        return fn(args)
    except Exception as e:  # noqa: BLE001
        return {"error": "%s: %s" % (type(e).__name__, e)}


def run_hist_traffic(args):
    """One quantized tree (graph form) on the synthetic workload, for a DRAM-traffic capture of the
    histogram kernel: prints its algorithmic bytes and launch count, the denominator of
    HIST_TRAFFIC_PER_BYTE (run under ncu with the dram__bytes_{read,write}.sum metrics and
    -k regex:k_hist_int, the capture's totals divided by these bytes)."""
    import torch
    from lgbm_gb300 import GpuTreeLearner
    ds, y, _ = build_dataset(args.rows)
    n = ds.num_data
    label = torch.from_numpy(y).cuda()
    learner = GpuTreeLearner(ds, make_cfg(True, args.leaves), loop_mode=1)
    score = torch.full((n,), float(y.astype(np.float64).mean()), dtype=torch.float64, device="cuda")
    gbuf, hbuf = learner.gradient_buffers()
    torch.cuda.synchronize()
    learner.objective_gradients(0, score.data_ptr(), label.data_ptr())
    learner.train_raw(gbuf, hbuf, on_device=True)
    torch.cuda.synchronize()
    tm = learner.last_timing()
    learner.close()
    return {"rows": n, "hist_launches": args.leaves - 1, "hist_alg_bytes": tm["hist_bytes"]}


def _shape_dict(shape, tuned):
    if shape is None:
        return None
    return {"hist_min_rows_per_cta": shape[0], "hist_ctas_per_feature_tile": shape[1], "partition_ctas": shape[2],
            "hist_direct_atomic_rows_per_cta": shape[3], "hist_ctas_per_cluster": shape[4],
            "source": "bk_learner_autotune" if tuned else "default"}


def _hist_launch_rows(splits, n, leaves, min_data=20):
    """Rows each histogram launch of one tree builds: the root's n, then the smaller child of each
    split when the children are searched (serial.rs:779-825: not when both have fewer than
    2 x min_data_in_leaf rows), else 0; a tree that stopped early leaves its last launches at 0."""
    rows = [n]
    for r in splits:
        lc, rc = int(r["left_count"]), int(r["right_count"])
        rows.append(0 if (lc < 2 * min_data and rc < 2 * min_data) else min(lc, rc))
    rows = rows[:leaves - 1]
    return rows + [0] * (leaves - 1 - len(rows))


def _roofline_by_leaf_size(launches, ds, n, peak):
    """The histogram launches grouped by the rows they build: algorithmic GB/s (the learner's
    per-row bytes: stored bins, a 4-bit tile's features half a byte; 2 packed bytes; 4 index bytes
    when gathered; the pool slot's bytes) over their CUDA-event time, and its fraction of `peak`."""
    feats = ds.features
    bin_bytes = 0.0
    for t0 in range(0, len(feats), 32):
        tile = feats[t0:t0 + 32]
        nib = all(fi.group_bins <= 16 for fi in tile)
        bin_bytes += len(tile) * (0.5 if nib else 1.0)
    slot = sum(fi.group_bins for fi in feats) * 8.0
    edges = [(n, n + 1, "root"), (1_000_000, n, "1M+"), (100_000, 1_000_000, "100k-1M"), (10_000, 100_000, "10k-100k"),
             (1, 10_000, "<10k")]
    out = []
    for lo, hi, name in edges:
        sel = [(r, t) for r, t in launches if lo <= r < hi and (r == n) == (name == "root")]
        if not sel:
            continue
        byt = sum(r * (bin_bytes + 2.0 + (0.0 if r == n else 4.0)) + slot for r, _ in sel)
        ms = sum(t for _, t in sel)
        gbs = byt / (ms * 1e6) if ms > 0 else None
        out.append({"leaf_rows": name, "launches": len(sel), "mean_us": round(1000.0 * ms / len(sel), 1),
                    "achieved_gbs": round(gbs, 1) if gbs else None,
                    "frac": round(gbs / peak, 4) if gbs else None})
    return out


def aggregate_ranks(ms_per_step, world):
    """Replicas: the slowest rank's time per step, and the iterations of all ranks per second."""
    ms = float(ms_per_step)
    if world > 1:
        import torch
        import torch.distributed as dist
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * 1000.0 / ms


def _device_view(ptr, count):
    """A float32 tensor view of a device buffer owned by the learner (CUDA array interface)."""
    import torch

    class _CAI:
        __cuda_array_interface__ = {"shape": (count,), "typestr": "<f4", "data": (int(ptr), False),
                                    "version": 3, "strides": None}
    return torch.as_tensor(_CAI(), device="cuda")


def _config(ds, args, world):
    """The workload both arms time (the same dict for the GPU arm and the CPU reference arm)."""
    return {"workload": WORKLOAD, "rows": ds.num_data, "features": ds.num_features, "num_leaves": args.leaves,
            "quantized": {"num_grad_quant_bins": 4, "stochastic_rounding": True},
            "parallelism": "replicas" if world > 1 else "one learner",
            "l2_flush": "inputs larger than L2 (stored bins %.2f GB)" % (ds.num_data * ds.num_features / 1e9)}


def _oracle_iterations(ds, y, quant, iters, warmup, threads, leaves=255, lr=0.1):
    """Boosting iterations of the oracle (the C++ port of the reference's tree learner) on all rows
    of a binned dataset, each timed whole: L2 gradients (objective/regression.rs:240-248), one
    tree (serial.rs:569-628, quantized or float path), shrinkage and the score update
    (serial.rs:1974-1990). `threads` host threads run the per-feature tasks and the block
    partition; the config's num_threads stays 16, the value that seeds the stochastic-rounding
    noise blocks of the GPU run (gradient_discretizer/mod.rs:87-106). Returns seconds per timed
    iteration and the final training L2."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import harness
    cfg = make_cfg(quant, leaves)
    orc = harness.OracleLearner(ds, cfg)
    orc.set_threads(threads)
    label = y.astype(np.float64)
    score = np.full(ds.num_data, float(np.mean(label)))
    h = np.ones(ds.num_data, np.float32)
    times = []
    for it in range(warmup + iters):
        t0 = time.perf_counter()
        g = (score - label).astype(np.float32)
        _, lv, _ = orc.train(g, h)
        if len(lv) > 1:
            vals = lv * lr
            vals[np.abs(vals) <= K_ZERO_THRESHOLD] = 0.0
            orc.add_score(vals, score)
        if it >= warmup:
            times.append(time.perf_counter() - t0)
    return times, float(np.mean((score - label) ** 2))


def cpu_baseline(ds, y, leaves=255):
    """The oracle on the GB300 machine's host cores: one quantized boosting iteration of the same
    workload (all rows), with every host thread."""
    threads = os.cpu_count() or 1
    times, _ = _oracle_iterations(ds, y, True, 1, 0, threads, leaves)
    return {"value": round(1.0 / times[0], 6), "unit": "iters/s", "cores": threads, "kind": "port",
            "sample": "one boosting iteration (L2 gradients + one quantized %d-leaf tree + score update) on all %d "
                      "rows of the workload, %.1f s" % (leaves, ds.num_data, times[0])}


def run_reference(args):
    """CPU arm: the oracle port of the reference's tree learner, with every host thread, on the
    whole workload — the same rows (binned by the oracle's own restatement of the reference's bin
    mappers, without the product library), the same quantized config as the GPU arm's `value`,
    every step a full boosting iteration. The float path of the oracle is timed beside it."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import harness
    from lgbm_gb300 import synthetic
    threads = os.cpu_count() or 1
    t0 = time.time()
    X, y = synthetic.l2_steps(n=args.rows, seed=0)
    ds = harness.bin_dense(X, max_bin=255, min_data_in_leaf=20, threads=threads)
    del X
    prep_s = time.time() - t0
    times, loss = _oracle_iterations(ds, y, True, args.steps, args.warmup, threads, args.leaves)
    ms = 1000.0 * float(np.mean(times))
    v = 1000.0 / ms
    ftimes, floss = _oracle_iterations(ds, y, False, min(args.steps, 2), 0, threads, args.leaves)
    return {"metric": METRIC, "impl": "reference", "value": round(v, 6), "unit": "iters/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int8 grad/hess, int64 histograms, f64 gains", "data": "synthetic (seeded)",
            "config": _config(ds, args, 1), "host_threads": threads,
            "cpu_baseline": {"value": round(v, 6), "unit": "iters/s", "cores": threads, "kind": "port",
                             "sample": "%d full boosting iterations (after %d untimed), all %d rows, quantized "
                                       "(the reference's quantized CPU path)" % (args.steps, args.warmup, ds.num_data)},
            "e2e": {"value": round(v, 6), "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "forms": {"quantized": {"iters_per_s": round(v, 6), "train_l2": loss},
                      "plain_float": {"iters_per_s": round(len(ftimes) / sum(ftimes), 6), "iterations": len(ftimes),
                                      "train_l2": floss}},
            "prep_s": round(prep_s, 1), "wall_s_timed": round(sum(times), 1)}


def main():
    # the batched-jobs form runs one stream per job: give the device more hardware queues than the
    # default 8 so that independent streams do not serialise behind each other
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--rows", type=int, default=10_000_000)
    ap.add_argument("--leaves", type=int, default=255)
    ap.add_argument("--batch-jobs", type=int, default=32,
                    help="independent jobs of the batched-jobs form (256 for the full set; 0: skip it)")
    ap.add_argument("--batch-iters", type=int, default=10, help="iterations per job of the batched-jobs form")
    ap.add_argument("--multiclass-rows", type=int, default=2_000_000,
                    help="rows of the K=10 multiclass form reported beside the headline (0: skip it)")
    ap.add_argument("--hist-traffic", action="store_true",
                    help="train one tree and print the histogram kernel's algorithmic bytes (for an ncu capture)")
    ap.add_argument("--autotune", type=int, default=1, help="1: autotune each form's launch shape first")
    ap.add_argument("--binary-rows", type=int, default=10_000_000,
                    help="rows of the 200-feature binary quantized form (0: skip it)")
    ap.add_argument("--only", choices=["multiclass", "batched", "binary"],
                    help="run only that side form and print its result (not a bench line)")
    args = ap.parse_args()
    if args.only:
        import torch
        torch.cuda.set_device(0)
        fn = {"multiclass": run_multiclass, "batched": run_batched_jobs, "binary": run_binary}[args.only]
        print(json.dumps(fn(args)))
        return
    if args.hist_traffic:
        print(json.dumps(run_hist_traffic(args)))
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    line = run_gpu(args, rank, world)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

"""Regenerates the golden fixtures in this folder from the bankai-lightgbm reference checkout.

Run in a container that has the reference at REFERENCE (default /root/reference):

    python tests/golden/make_golden.py [REFERENCE]

It copies, unchanged, the reference's own golden data for the tree-learner path:

* ``train/<case>/{x.npy,y.npy[,w.npy],params.json,model.txt}`` — upstream-LightGBM 4.7.0 models that the
  reference reproduces byte for byte (tests/fixtures/train, generated on darwin/arm64 with
  ``deterministic, num_threads=1, force_col_wise, seed=7``), for the cases inside this learner's
  scope (dense numerical and categorical features, L2 / binary / multiclass objectives; plain
  bagging and the by-tree feature fraction, which reach the learner as its `rows` and
  feature-mask inputs);
* ``train_oracle/<case>/`` — the same files for 31 cases that differ from those only on the
  Trainer's side of the learner (binary sigmoid 0.7 with scale_pos_weight 2.5, is_unbalance,
  bagging balanced by label, reg_sqrt, huber, fair, poisson, gamma, tweedie, cross_entropy,
  cross_entropy_lambda, one-vs-all multiclass, and the leaf-renewing l1, quantile and mape,
  weighted and not; random-forest boosting), pinned on
  the oracle; where the reference keeps the model its linux-x86_64 build gives (unfused madd,
  glibc's libm) as ``model.linux-x86_64.txt``, that file comes too;
* ``quantized_gradients.json`` — 16 upstream stumps for the gradient discretizer
  (tests/fixtures/quantized_gradients.json);
* ``predict/<case>/`` — six upstream models with their training / test rows, the leaf index of
  every test row in every tree and the raw scores (tests/fixtures/{binary, missing, zero_as_missing, regression_l2,
  categorical, multiclass});
* ``metrics/{binary, reg, multiclass}/`` — scores, labels and upstream's metric values
  (tests/fixtures/metrics), for the benchmark's held-out metrics;
* ``datasets/<case>.json`` + ``datasets/x_*.npz`` — the 20 upstream dataset cases of
  tests/fixtures/datasets: the value matrix and the bin mappers upstream's ``save_binary`` wrote
  for it (read from its dataset.bin as the reference's io/binary.rs reads it);

and extracts the known-answer vectors that the reference keeps inside its Rust tests:

* ``vectors.json`` — the std::mt19937 / libc++ distribution draws
  (crates/lgbm-core/tests/mt19937.rs), the nearest-rounding packed values
  (crates/lgbm-core/tests/quantized_gradients.rs:99-138) and the integer split-search
  histograms (crates/lgbm-core/tests/quantized_split_search.rs:186-223).

Nothing at test time reads the reference; the tests read only this folder.
"""
import hashlib
import json
import os
import re
import shutil
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["binary", "l2_default", "l2_nan", "l2_zero", "l2_zero_as_missing", "l2_small", "l2_regularized",
         "l2_max_delta_smooth", "l2_max_depth", "l2_no_boost_from_average", "multiclass", "bagging",
         "bagging_no_freq", "bagging_feature_fraction", "feature_fraction", "cat_default", "cat_binary", "cat_nan",
         "cat_onehot", "cat_regularized", "cat_bagging", "l2_default_weighted", "binary_weighted",
         "multiclass_weighted", "bagging_weighted", "cat_default_weighted", "feature_fraction_bynode",
         "feature_fraction_both", "goss", "goss_dense_sample", "goss_weighted", "interaction", "interaction_bynode",
         "interaction_sampled"]
# Cases whose differences lie on the Trainer's side of the learner only (the binary objective's
# sigmoid and label weights, bagging balanced by label, the gradient-only regression and
# cross-entropy objectives): copied to train_oracle/ and pinned on the oracle; the learner receives
# the same kind of gradients and row lists as in the cases above.
ORACLE_CASES = ["binary_sigmoid", "binary_unbalance", "bagging_balanced", "l2_sqrt", "huber", "huber_weighted",
                "fair", "fair_weighted", "poisson", "poisson_weighted", "gamma", "gamma_weighted", "tweedie",
                "tweedie_weighted", "xentropy", "xentropy_weighted", "xentlambda", "xentlambda_weighted", "l1",
                "l1_weighted", "l1_no_boost_from_average", "quantile", "quantile_high", "quantile_weighted", "mape",
                "mape_weighted", "multiclassova", "multiclassova_weighted", "rf", "rf_binary", "rf_feature_fraction"]


# ---- upstream binary dataset files (the reference's io/binary.rs reader, restated) ----
_TOKEN = b"______LightGBM_Binary_File_Token______\n"


class _Reader:
    """Little-endian reader of upstream's 8-byte aligned layout (io/binary.rs:13-89)."""

    def __init__(self, buf):
        self.buf, self.pos = buf, 0

    def take(self, n):
        s = self.buf[self.pos:self.pos + n]
        assert len(s) == n, "binary dataset truncated"
        self.pos += n
        return s

    def i32(self):
        return struct.unpack("<i", self.take(4))[0]

    def f64(self):
        return struct.unpack("<d", self.take(8))[0]

    def u64(self):
        return struct.unpack("<Q", self.take(8))[0]

    def aligned_i32(self):
        v = self.i32()
        self.take(4)
        return v

    def aligned_bool(self):
        return self.take(8)[0] != 0

    def aligned_i32_vec(self, n):
        start = self.pos
        v = [self.i32() for _ in range(n)]
        used = self.pos - start
        self.take((used + 7) // 8 * 8 - used)
        return v

    def aligned_bytes(self, n):
        s = self.take(n)
        self.take((n + 7) // 8 * 8 - n)
        return s


def _bin_mapper(r):
    """BinMapper::from_bytes (io/bin.rs:666-703)."""
    m = {"num_bin": r.aligned_i32(), "missing_type": r.aligned_i32(), "is_trivial": r.aligned_bool(),
         "sparse_rate": r.f64(), "bin_type": r.aligned_i32(), "min_val": r.f64(), "max_val": r.f64(),
         "default_bin": r.aligned_i32(), "most_freq_bin": r.aligned_i32()}
    if m["bin_type"] == 0:
        m["bin_upper_bound"] = [r.f64() for _ in range(m["num_bin"])]
    else:
        m["bin_2_categorical"] = [r.i32() for _ in range(m["num_bin"])]
    return m


def read_bin_mappers(path):
    """The used-feature map and every used feature's BinMapper of an upstream binary dataset file
    (io/binary.rs:146-295: token, header, metadata, feature groups)."""
    r = _Reader(open(path, "rb").read())
    assert r.aligned_bytes(len(_TOKEN)) == _TOKEN
    header_size = r.u64()
    h0 = r.pos
    num_data, num_features, ntf = r.aligned_i32(), r.aligned_i32(), r.aligned_i32()
    for _ in range(4):  # label_idx, max_bin, bin_construct_sample_cnt, min_data_in_bin
        r.aligned_i32()
    for _ in range(3):  # use_missing, zero_as_missing, has_raw
        r.aligned_bool()
    used_feature_map = r.aligned_i32_vec(ntf)
    num_groups = r.aligned_i32()
    r.aligned_i32_vec(num_features)  # real_feature_idx
    feature2group = r.aligned_i32_vec(num_features)
    feature2subfeature = r.aligned_i32_vec(num_features)
    r.pos = h0 + header_size  # the rest of the header (bin boundaries, names, forced bins)
    meta_size = r.u64()
    r.pos += meta_size
    groups = []
    for _ in range(num_groups):
        size = r.u64()
        start = r.pos
        for _ in range(3):  # is_multi_val, is_dense_multi_val, is_sparse
            r.aligned_bool()
        nfeat = r.aligned_i32()
        groups.append([_bin_mapper(r) for _ in range(nfeat)])
        r.pos = start + size
    mappers = []
    for real in range(ntf):
        inner = used_feature_map[real]
        if inner < 0:
            mappers.append(None)
        else:
            mappers.append(groups[feature2group[inner]][feature2subfeature[inner]])
    return {"num_data": num_data, "mappers": mappers}


def copy_datasets(fx):
    """tests/fixtures/datasets: the value matrix of each case (deduplicated, compressed) and the
    bin mappers upstream wrote into its dataset.bin, as JSON."""
    src_root = os.path.join(fx, "datasets")
    dst_root = os.path.join(HERE, "datasets")
    os.makedirs(dst_root, exist_ok=True)
    for case in sorted(os.listdir(src_root)):
        src = os.path.join(src_root, case)
        x = np.load(os.path.join(src, "x.npy"))
        xname = "x_%s.npz" % hashlib.sha256(x.tobytes()).hexdigest()[:12]
        if not os.path.exists(os.path.join(dst_root, xname)):
            np.savez_compressed(os.path.join(dst_root, xname), x=x)
        P = json.load(open(os.path.join(src, "params.json")))
        P["x"] = xname
        P.update(read_bin_mappers(os.path.join(src, "dataset.bin")))
        with open(os.path.join(dst_root, case + ".json"), "w") as f:
            json.dump(P, f)


PREDICT_CASES = ["binary", "missing", "zero_as_missing", "regression_l2", "categorical", "multiclass"]


METRIC_CASES = ["binary", "reg", "multiclass"]


def copy_metric_cases(fx):
    """tests/fixtures/metrics/{binary, reg, multiclass}: scores, labels and upstream's metric
    values at those scores."""
    for case in METRIC_CASES:
        src = os.path.join(fx, "metrics", case)
        dst = os.path.join(HERE, "metrics", case)
        os.makedirs(dst, exist_ok=True)
        for name in ("score.npy", "label.npy", "params.json", "expected.json"):
            shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))


def copy_predict_cases(fx):
    """tests/fixtures/<case>: an upstream model, its training and test rows and the leaf every test
    row reaches in every tree (pred_leaf.npy), for the routing of held-out rows."""
    for case in PREDICT_CASES:
        src = os.path.join(fx, case)
        dst = os.path.join(HERE, "predict", case)
        os.makedirs(dst, exist_ok=True)
        for name in ("train.npy", "test.npy", "pred_leaf.npy", "pred_raw.npy", "model.txt", "params.json"):
            shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))


def _ints(text):
    return [int(x) for x in re.findall(r"-?\d+", text)]


def main(ref):
    fx = os.path.join(ref, "tests", "fixtures")
    for case, sub in [(c, "train") for c in CASES] + [(c, "train_oracle") for c in ORACLE_CASES]:
        src = os.path.join(fx, "train", case)
        dst = os.path.join(HERE, sub, case)
        os.makedirs(dst, exist_ok=True)
        for name in ("x.npy", "y.npy", "w.npy", "params.json", "model.txt", "model.linux-x86_64.txt"):
            if name in ("w.npy", "model.linux-x86_64.txt") and not os.path.exists(os.path.join(src, name)):
                continue  # sample weights, and the linux-x86_64 libm variant, only where the case has them
            shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))
    shutil.copyfile(os.path.join(fx, "quantized_gradients.json"), os.path.join(HERE, "quantized_gradients.json"))
    copy_datasets(fx)
    copy_predict_cases(fx)
    copy_metric_cases(fx)

    tests = os.path.join(ref, "crates", "lgbm-core", "tests")
    mt = open(os.path.join(tests, "mt19937.rs")).read()
    vec = {}
    m = re.search(r"assert_eq!\(value, ([\d_]+)\)", mt)
    vec["mt19937_default_10000th"] = int(m.group(1).replace("_", ""))
    m = re.search(r"std::mt19937\((\d+)\), std::uniform_real_distribution.*?= \[([^\]]*)\];", mt, re.S)
    vec["uniform_real_01"] = {"seed": int(m.group(1)),
                              "bits": [int(x, 16) for x in re.findall(r"0x([0-9a-f]+)", m.group(2))]}
    m = re.search(r"Mt19937::new\((\d+)\);\s*for want in \[([^\]]*)\]\s*\{\s*assert_eq!\(e\.uniform_int_inclusive\((\d+)\)",
                  mt)
    ui = [{"seed": int(m.group(1)), "n": int(m.group(3)), "draws": _ints(m.group(2))}]
    for m in re.finditer(r"let mut (e\d+) = Mt19937::new\((\d+)\);\s*for want in \[([^\]]*)\]\s*\{\s*"
                         r"assert_eq!\(\1\.uniform_int_inclusive\((\d+)\)", mt):
        ui.append({"seed": int(m.group(2)), "n": int(m.group(4)), "draws": _ints(m.group(3))})
    vec["uniform_int_inclusive"] = ui

    qg_all = open(os.path.join(tests, "quantized_gradients.rs")).read()
    qg = qg_all[qg_all.index("fn quantized_nearest_reuses_buffer_and_recomputes_scales"):]
    qg = qg[:qg.index("#[test]")]
    nearest = []
    for m in re.finditer(r"discretize_nearest\(&\[([^\]]*)\], &\[([^\]]*)\]\)\s*\.unwrap\(\);.*?"
                         r"packed_gradients_hessians\(\), &\[([^\]]*)\]\);\s*assert_eq!\(q\.gradient_scale\(\), "
                         r"([\d.]+)\);\s*assert_eq!\(q\.hessian_scale\(\), ([\d.]+)\);", qg, re.S):
        g = [float(x) for x in m.group(1).split(",")]
        hs = m.group(2).strip()
        if ";" in hs:
            val, cnt = hs.split(";")
            h = [float(val)] * int(cnt)
        else:
            h = [float(x) for x in hs.split(",")]
        nearest.append({"gradients": g, "hessians": h, "packed": _ints(m.group(3)),
                        "gradient_scale": float(m.group(4)), "hessian_scale": float(m.group(5))})
    head = re.search(r"GradientDiscretizer::new\(5, 4, false\)", qg)
    vec["nearest_bins4"] = nearest if head else []
    qg = qg_all
    m = re.search(r"new\(2, 4, true\).*?discretize_nearest\(&\[([^\]]*)\], &\[0\.0; 2\]\).*?"
                  r"packed_gradients_hessians\(\), &\[([^\]]*)\]\);", qg, re.S)
    vec["nearest_const_hess_bins4"] = {"gradients": [float(x) for x in m.group(1).split(",")],
                                       "hessians": [0.0, 0.0], "packed": _ints(m.group(2))}

    qs = open(os.path.join(tests, "quantized_split_search.rs")).read()
    hists = []
    for m in re.finditer(r"let hist = \[(.*?)\];(.*?)\n\}", qs, re.S):
        pairs = re.findall(r"\((-?\d+)i?6?4?,\s*(-?\d+)i?6?4?\)", m.group(1))
        checks = re.findall(r"check\(&hist, ([\d.]+), ([\d.]+), ([\d.]+), (\d+)\)", m.group(2))
        hists.append({"hist": [[int(a), int(b)] for a, b in pairs],
                      "checks": [[float(a), float(b), float(c), int(d)] for a, b, c, d in checks]})
    vec["int_split_search"] = hists
    with open(os.path.join(HERE, "vectors.json"), "w") as f:
        json.dump(vec, f, indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")

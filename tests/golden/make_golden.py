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
* ``quantized_gradients.json`` — 16 upstream stumps for the gradient discretizer
  (tests/fixtures/quantized_gradients.json);

and extracts the known-answer vectors that the reference keeps inside its Rust tests:

* ``vectors.json`` — the std::mt19937 / libc++ distribution draws
  (crates/lgbm-core/tests/mt19937.rs), the nearest-rounding packed values
  (crates/lgbm-core/tests/quantized_gradients.rs:99-138) and the integer split-search
  histograms (crates/lgbm-core/tests/quantized_split_search.rs:186-223).

Nothing at test time reads the reference; the tests read only this folder.
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["binary", "l2_default", "l2_nan", "l2_zero", "l2_zero_as_missing", "l2_small", "l2_regularized",
         "l2_max_delta_smooth", "l2_max_depth", "l2_no_boost_from_average", "multiclass", "bagging",
         "bagging_no_freq", "bagging_feature_fraction", "feature_fraction", "cat_default", "cat_binary", "cat_nan",
         "cat_onehot", "cat_regularized", "cat_bagging", "l2_default_weighted", "binary_weighted",
         "multiclass_weighted", "bagging_weighted", "cat_default_weighted", "feature_fraction_bynode",
         "feature_fraction_both", "goss", "goss_dense_sample", "goss_weighted"]


def _ints(text):
    return [int(x) for x in re.findall(r"-?\d+", text)]


def main(ref):
    fx = os.path.join(ref, "tests", "fixtures")
    for case in CASES:
        src = os.path.join(fx, "train", case)
        dst = os.path.join(HERE, "train", case)
        os.makedirs(dst, exist_ok=True)
        for name in ("x.npy", "y.npy", "w.npy", "params.json", "model.txt"):
            if name == "w.npy" and not os.path.exists(os.path.join(src, name)):
                continue  # sample weights only where the case has them
            shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))
    shutil.copyfile(os.path.join(fx, "quantized_gradients.json"), os.path.join(HERE, "quantized_gradients.json"))

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

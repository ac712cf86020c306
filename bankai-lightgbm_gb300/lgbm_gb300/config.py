"""Learner configuration (the ``bk_config`` record of include/bkgpu.h).

Field meanings and defaults follow bankai-lightgbm's ``Config`` (crates/lgbm-core/src/config/
auto.rs:174-251) for the parameters the tree learner reads.
"""
import numpy as np

CONFIG_DTYPE = np.dtype([
    ("num_leaves", np.int32), ("max_depth", np.int32), ("min_data_in_leaf", np.int32), ("_pad0", np.int32),
    ("min_sum_hessian_in_leaf", np.float64), ("lambda_l1", np.float64), ("lambda_l2", np.float64),
    ("max_delta_step", np.float64), ("path_smooth", np.float64), ("min_gain_to_split", np.float64),
    ("use_quantized_grad", np.int32), ("num_grad_quant_bins", np.int32), ("quant_train_renew_leaf", np.int32),
    ("stochastic_rounding", np.int32), ("seed", np.int32), ("num_threads", np.int32), ("fused_madd", np.int32),
    ("is_constant_hessian", np.int32), ("max_cat_to_onehot", np.int32), ("max_cat_threshold", np.int32),
    ("cat_smooth", np.float64), ("cat_l2", np.float64), ("min_data_per_group", np.int32), ("_pad1", np.int32),
], align=True)

DEFAULTS = dict(num_leaves=31, max_depth=-1, min_data_in_leaf=20, min_sum_hessian_in_leaf=1e-3, lambda_l1=0.0,
                lambda_l2=0.0, max_delta_step=0.0, path_smooth=0.0, min_gain_to_split=0.0, use_quantized_grad=0,
                num_grad_quant_bins=4, quant_train_renew_leaf=0, stochastic_rounding=1, seed=0, num_threads=1,
                fused_madd=0, is_constant_hessian=0, max_cat_to_onehot=4, max_cat_threshold=32, cat_smooth=10.0,
                cat_l2=10.0, min_data_per_group=100)

_ALIASES = {"min_child_samples": "min_data_in_leaf", "min_child_weight": "min_sum_hessian_in_leaf",
            "reg_alpha": "lambda_l1", "reg_lambda": "lambda_l2", "min_split_gain": "min_gain_to_split",
            "num_leaf": "num_leaves", "max_leaves": "num_leaves", "random_state": "seed",
            "random_seed": "seed", "n_jobs": "num_threads"}


class LearnerConfig:
    def __init__(self, **kw):
        self.values = dict(DEFAULTS)
        for k, v in kw.items():
            k = _ALIASES.get(k, k)
            if k in self.values:
                self.values[k] = v

    def __getattr__(self, k):
        try:
            return self.__dict__["values"][k]
        except KeyError:
            raise AttributeError(k)

    def record(self):
        arr = np.zeros(1, dtype=CONFIG_DTYPE)
        for k, v in self.values.items():
            arr[k] = v
        return arr

"""GB300-native tree learner for bankai-lightgbm's histogram hot path.

Host-side mirror of the reference's ``SerialTreeLearner`` (crates/lgbm-core/src/treelearner/
serial.rs) over the C-ABI library ``lib/libbkgpu.so`` (declared in ``include/bkgpu.h``).
"""
from .dataset import BinnedDataset, FeatureInfo, FEATURE_DTYPE  # noqa: F401
from .tree import Tree, SPLIT_DTYPE  # noqa: F401
from .config import LearnerConfig, CONFIG_DTYPE  # noqa: F401
from .learner import GpuTreeLearner, LearnerGroup, train_batch  # noqa: F401

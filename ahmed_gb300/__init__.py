"""GB300-native H-matrix hot path: ACA assembly, H-matvec and GMRES/CG on sm_103a.

The compute path is libahx.so (hand-written CUDA kernels behind a C ABI,
include/ahx.h); this package is the host-side mirror of the reference's
interface.
"""
from . import geometry  # noqa: F401
from .hmatrix import (  # noqa: F401
    CG,
    GMRes,
    HBatch,
    HMatrix,
    loadmbls,
    matgenGeH_omp,
    mbls_header,
    mean_nn,
    min_nn,
    mltaGeHGeM,
    mltaGeHVec,
    savembls,
)
from ._capi import BF16_FP32, DF64, FP32, FP64, TREE_BBX, TREE_PCA, lib  # noqa: F401
from .rank_predictor import RankPredictor, training_set  # noqa: F401

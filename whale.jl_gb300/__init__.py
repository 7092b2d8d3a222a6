"""GB300-native Whale likelihood: the amalgamated reconciliation likelihood of
gene-family CCDs under the duplication-loss + WGD model, evaluated on one
GB300 by hand-written sm_103a CUDA kernels behind a C ABI (libwhalegpu).

The Python layer mirrors the reference's Julia API (Whale.jl v2.1.0,
src/Whale.jl:38-39): ``WhaleModel``, ``DLWGD``, ``ConstantDLWGD``, ``CCD``,
``read_ale``, ``logpdf``, ``logpdf_inplace`` (``logpdf!``), ``loglikelihood``,
plus ``gradient``/``logpdf_gradient`` in place of ForwardDiff over the rates,
the multi-model forms ``MixtureModel`` / ``ModelArray`` (src/core.jl:66-79)
and ``backtrack`` (reconciled-tree sampling, src/track.jl:180-488).
Tree helpers follow NewickTree: ``readnw``, ``insertnode`` (``insertnode!``),
``getlca``, ``postwalk``, ``extree``.
"""
from ._native import WhaleError
from .ccd import CCD, parse_ale_text, read_ale
from .core import (Batch, Context, default_context, get_batch, gradient, logpdf, logpdf_gradient, logpdf_inplace,
                   logpdf_plain, loglikelihood, map_gradient, nowhere_condition)
from .mixture import MixtureModel, ModelArray
from .autotune import tune
from .track import RecNode, RecTree, TrackSummary, backtrack, getpairs, sumtrees, track
from .model import (ConstantDLWGD, DLWGD, NoCondition, NonExtinctCondition, NowhereExtinctCondition, RootCondition,
                    WhaleModel, condition)
from .newick import (EXTREE, Node, addbranchwgds, copytree, extree, getlca, getleaves, getroot, insertnode, nwstr,
                     postwalk, prewalk, readnw)

logpdf_ = logpdf_inplace

__all__ = [
    "WhaleModel", "DLWGD", "ConstantDLWGD", "RootCondition", "NonExtinctCondition", "NoCondition",
    "NowhereExtinctCondition", "condition", "nowhere_condition",
    "CCD", "read_ale", "parse_ale_text", "logpdf", "logpdf_inplace", "logpdf_", "loglikelihood", "gradient",
    "logpdf_gradient", "logpdf_plain", "map_gradient", "Batch", "Context", "default_context", "get_batch",
    "readnw", "nwstr", "insertnode", "getlca", "getleaves", "getroot", "postwalk", "prewalk", "extree", "EXTREE",
    "addbranchwgds", "copytree", "Node", "WhaleError", "MixtureModel", "ModelArray", "backtrack", "track", "sumtrees", "getpairs", "TrackSummary", "RecNode",
    "RecTree", "tune",
]

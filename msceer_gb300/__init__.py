"""GB300-native (sm_103a) discrete-gradient engine with MSCEER's .grad semantics.

The compute path is libmsc_gpu.so (hand-written CUDA behind a C ABI, see
include/msc_gpu.h); this package is the host-side mirror of the reference's
interface for the path (TopologicalRegularGrid3D / DiscreteGradientLabeling and
the steepest_lstar entry) plus the synthetic workload generators.
"""
from .api import (  # noqa: F401
    DiscreteGradientLabeling,
    TopologicalRegularGrid2D,
    TopologicalRegularGrid3D,
    ascending_manifold_dims,
    clean_regions,
    conforming_grad,
    integrated_labels,
    integrated_labels_batch,
    lower_star_grad,
    lower_star_grad_batch,
    lower_star_pairs,
    ms_graph,
    num_cells,
    saddle_lines,
    steepest_lstar,
)

__version__ = "0.1.0"

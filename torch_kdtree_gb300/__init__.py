"""GB300-native exact KNN engine with torch_kdtree's API.

    from torch_kdtree_gb300 import build_kd_tree
    tree = build_kd_tree(points_ref)            # on a CUDA device
    dists, inds = tree.query(points_query, nr_nns_searches=k)
"""
from .nn_distance import (TorchKDTree, build_kd_tree, default_levels, gpu_available, load_kd_tree, nn_distance,
                          nn_distance_bidirectional)

__all__ = ["build_kd_tree", "gpu_available", "TorchKDTree", "default_levels", "load_kd_tree", "nn_distance",
           "nn_distance_bidirectional"]
__version__ = "0.1.0"

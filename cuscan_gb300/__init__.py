"""cuscan_gb300: GB300-native (sm_103a) exact HDBSCAN fit core.

The product is the C-ABI shared library built from ``csrc/`` (declared in
``include/cuscan_gb300.h``); this package loads it with ctypes and exposes the
``HDBSCAN`` estimator surface of cuscan. There is no CPU fallback.
"""
from ._lib import Context, clusters_from_spanning_tree, dbscan_cut, load, library_path
from .hdbscan import HDBSCAN, context, fit_hdbscan
from .prediction import HDBSCANPredictor
from .serving import FitServer

__all__ = ["HDBSCAN", "HDBSCANPredictor", "FitServer", "Context", "context", "fit_hdbscan",
           "clusters_from_spanning_tree", "dbscan_cut", "load", "library_path"]
__version__ = "0.1.0"

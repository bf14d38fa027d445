"""GB300 exact k-NN kd-tree with the API of FujishigeTemma/kdtree-rs.

`from kdtree import KDTree` as in the reference (python/kdtree/__init__.py:1-3).
"""
from ._core import BatchQuery, KDTree, Server

__all__ = ["KDTree", "BatchQuery", "Server"]

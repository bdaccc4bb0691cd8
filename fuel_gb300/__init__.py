"""fuel_gb300 -- GB300-native engine for kno10/fuel's linear-scan kNN / range
search and Lloyd k-means hot path.

``fuel_gb300.search`` and ``fuel_gb300.cluster`` mirror ``fuel.search`` and
``fuel.cluster.kmeans``; the compute runs in libfuelg.so (hand-written
sm_103a CUDA behind the C ABI of include/fuelg.h).
"""
from .search import SearchIndex, knn_batched, knn_search, pairwise_distances, range_search  # noqa: F401
from .cluster import KMeansResult, kmeans, kmeans_batched, lloyd_assign  # noqa: F401

__version__ = "0.1.0"

"""Discretization API (pyemma.coordinates): cluster_kmeans, assign_to_centers."""
from .api import assign_to_centers, cluster_kmeans
from .clustering import AssignCenters, KmeansClustering

__all__ = ["assign_to_centers", "cluster_kmeans", "AssignCenters", "KmeansClustering"]

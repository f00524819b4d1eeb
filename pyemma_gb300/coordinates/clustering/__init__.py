"""Clustering estimators (pyemma.coordinates.clustering)."""
from .assign import AssignCenters
from .interface import AbstractClustering
from .kmeans import KmeansClustering

__all__ = ["AbstractClustering", "AssignCenters", "KmeansClustering"]

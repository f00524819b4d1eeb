"""Clustering estimators (pyemma.coordinates.clustering)."""
from .assign import AssignCenters
from .interface import AbstractClustering
from .kmeans import KmeansClustering, MiniBatchKmeansClustering
from .regspace import NotConvergedWarning, RegularSpaceClustering
from .uniform_time import UniformTimeClustering

__all__ = ["AbstractClustering", "AssignCenters", "KmeansClustering", "MiniBatchKmeansClustering",
           "RegularSpaceClustering", "UniformTimeClustering", "NotConvergedWarning"]

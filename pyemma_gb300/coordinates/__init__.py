"""Discretization API (pyemma.coordinates): cluster_kmeans, assign_to_centers and the sibling estimators."""
from .api import (assign_to_centers, cluster_kmeans, cluster_mini_batch_kmeans, cluster_regspace,
                  cluster_uniform_time)
from .clustering import (AssignCenters, KmeansClustering, MiniBatchKmeansClustering, RegularSpaceClustering,
                         UniformTimeClustering)

__all__ = ["assign_to_centers", "cluster_kmeans", "cluster_mini_batch_kmeans", "cluster_regspace",
           "cluster_uniform_time", "AssignCenters", "KmeansClustering", "MiniBatchKmeansClustering",
           "RegularSpaceClustering", "UniformTimeClustering"]

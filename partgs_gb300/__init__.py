"""GB300-native differentiable 2D-Gaussian surfel rasteriser for PartGS.

Submodules:
  diff_surfel_rasterization        drop-in for the reference's plain rasteriser API
  diff_surfel_rasterization_part   drop-in for the part-map variant
  batched                          many views / many scenes in one launch sequence
  binding                          superquadric -> surfel binding with a hand-written adjoint
  scenes, cameras                  seeded synthetic workloads
"""
__version__ = "0.1.0"

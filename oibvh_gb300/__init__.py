"""oibvh_gb300: the oibvh collision pipeline (build, refit, BVTT broad phase,
triangle narrow phase) as hand-written sm_103a CUDA kernels behind a C ABI
(include/oibvh_gb300.h), with a Python mirror of the reference's
OibvhTree / Scene interface."""
from .api import DeviceType, OibvhError, OibvhTree, Scene, Server
from .meshes import Mesh

__all__ = ["DeviceType", "OibvhError", "OibvhTree", "Scene", "Server", "Mesh"]

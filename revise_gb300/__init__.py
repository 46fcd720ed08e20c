"""revise_gb300: GB300-native (sm_103a) sparse-octree interpolation, block ray
casting and image-part blending for ReVisE block trees, behind the s3r C ABI
(include/s3r.h).  Build the library with `python -m revise_gb300.build`."""
from . import _lib, host, workloads  # noqa: F401

__all__ = ["_lib", "host", "workloads"]

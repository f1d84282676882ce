"""doonengine_gb300 -- DoonEngine's per-voxel lighting and draw path on GB300 (CUDA sm_103a).

The product is ``libdoonengine.so`` (built in-tree under ``doonengine_gb300/_build``): the DN_* C API of
``include/DoonEngine/voxel.h`` over the ``dn_cuda_*`` C ABI of ``include/dn_cuda.h``.  This package
builds and loads it and mirrors the API for Python callers; all compute runs in the CUDA kernels and
there is no CPU fallback (operations on a machine without a GPU fail with an error).
"""
from . import build as _build_mod
from ._lib import load, library_path, check_layout, exported_names
from .volume import Volume, Image, Texture, Batch, Server, init, install_message_callback, messages, DN_READ, DN_WRITE, DN_READ_WRITE


def build(force=False):
    """Compile libdoonengine.so for sm_103a (in-tree) and return its path."""
    return _build_mod.build(force=force)


__all__ = ["build", "load", "library_path", "check_layout", "exported_names", "Volume", "Image", "Texture", "Batch", "Server", "init",
           "install_message_callback", "messages", "DN_READ", "DN_WRITE", "DN_READ_WRITE"]

"""jetshow_gb300 -- GB300 (sm_103a) renderer of jetshow's per-pixel polarised
synchrotron transfer path, behind jetshow's model classes (``jet``), its
``pyjetshow`` binding (``pyjetshow``) and a C ABI (``include/jetshow_capi.h``).

The compute runs only in the in-tree CUDA library
``jetshow_gb300/_build/libjetshow_gb300.so``; importing a symbol that needs
it raises if it has not been built (``jetshow_gb300.build.build()``).
"""
from . import _capi  # noqa: F401
from .runtime import Context, JetshowError, default_context, mas_to_pc  # noqa: F401

__all__ = ["Context", "JetshowError", "default_context", "mas_to_pc"]

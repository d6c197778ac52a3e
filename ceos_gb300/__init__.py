"""GB300-native (sm_103a) CEOs / coCEOs / streamCEOs index.

``ceos_gb300.CEOs`` is the drop-in module (classes ``CEOs`` and
``streamCEOs``); ``ceos_gb300.build`` compiles the CUDA library in-tree;
``ceos_gb300.serving`` runs the continuous-batching request loop.
"""
from . import _capi  # noqa: F401

__version__ = "0.1.0"


def library_path() -> str:
    return _capi.LIB_PATH

"""GB300-native engine for the finite-difference hot path of PseudoAcousticModeling.

The compute path is hand-written sm_103a CUDA behind the C ABI of
include/pam.h (library built in-tree by ``build.build()``); ``Engine`` is its
Python handle, and ``survey``, ``modeling``, ``migration`` and ``inversion``
mirror the reference's own classes on top of it.
"""
from .engine import Config, Engine  # noqa: F401
from ._lib import PamError  # noqa: F401

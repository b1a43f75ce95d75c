"""linon_gb300 — GB300-native nonlinear ray casting (the hot path of linon).

The engine lives in liblinon.so (C ABI: include/linon.h); this package is the
Python host side: ctypes bindings, scene/camera builders, the MainView
mirror and the benchmark workloads.
"""
from ._abi import (Camera, LinonCompileError, LinonError, MarchParams, RaySample, Settings,
                   FIELD_IDS, load, reference_params)
from .engine import (Engine, Field, FramePlanes, outline_indices, predefined_name, predefined_source,
                     translate_wgsl, validate_field)

__all__ = ["Camera", "Engine", "Field", "FramePlanes", "LinonCompileError", "LinonError", "MarchParams",
           "RaySample", "Settings", "FIELD_IDS", "load", "outline_indices", "predefined_name",
           "predefined_source", "reference_params", "translate_wgsl", "validate_field"]

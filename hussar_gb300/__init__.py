"""hussar_gb300: libhussar's Monte Carlo radar integrator on one NVIDIA GB300.

The compute path is libhsr_gb300.so (hand-written sm_103a CUDA behind the C ABI in
include/hsr_gb300.h). This package mirrors libhussar's Scene/Sensor/Integrator API
and libradar's FMCW types on top of it. There is no CPU fallback.
"""
from . import io, radar, scenes, serve
from ._lib import (HSR_PHASE_REFERENCE_FP32, HSR_PHASE_SPLIT_FP64, HSR_SPLAT_DIRICHLET16, HSR_SPLAT_FINE_SYNTH,
                   HsrError)
from .core import AWRAngularDistribution, FFAntenna, NFAntenna, PathTracer, Scene, TriangleMesh, gb300
from .radar import Frame, FrameConfig, RFConfig
from .serve import Server

__all__ = ["io", "radar", "scenes", "serve", "Server", "RFConfig", "FrameConfig", "Frame", "TriangleMesh", "NFAntenna", "FFAntenna",
           "AWRAngularDistribution", "Scene", "PathTracer", "gb300", "HsrError", "HSR_PHASE_REFERENCE_FP32",
           "HSR_PHASE_SPLIT_FP64", "HSR_SPLAT_DIRICHLET16", "HSR_SPLAT_FINE_SYNTH"]

"""Drop-in replacement for the reference's ``fastqslpy`` package
(fastqslpy/__init__.py:1-5) on GB300.

    import fastqsl_gb300.fastqslpy as fastqslpy
    TraceAllBline = fastqslpy.kernels.compileTraceBlineAdaptive()
    TraceAllBline(blck, grd, (Bx_gpu, By_gpu, ...))   # same 35 arguments
    Q = fastqslpy.FastQSL.QCalcPlane(...)

``kernels``, ``FastQSL`` and ``MagTool`` keep the reference's entry points
and argument lists; arrays may be PyTorch CUDA tensors or CuPy arrays
(``MagTool`` also takes the NumPy arrays its reference takes and returns
NumPy arrays, as there).
"""
from . import FastQSL, MagTool, kernels

__all__ = ["kernels", "FastQSL", "MagTool"]

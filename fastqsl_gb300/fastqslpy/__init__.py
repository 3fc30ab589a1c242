"""Drop-in replacement for the reference's ``fastqslpy`` package
(fastqslpy/__init__.py:1-5) on GB300.

    import fastqsl_gb300.fastqslpy as fastqslpy
    TraceAllBline = fastqslpy.kernels.compileTraceBlineAdaptive()
    TraceAllBline(blck, grd, (Bx_gpu, By_gpu, ...))   # same 35 arguments
    Q = fastqslpy.FastQSL.QCalcPlane(...)

``kernels`` and ``FastQSL`` keep the reference's entry points and argument
lists; arrays may be PyTorch CUDA tensors or CuPy arrays.  The reference's
``MagTool`` (a NumPy toy tracer that nothing in the package calls) is not
part of the GPU path and is not provided.
"""
from . import FastQSL, kernels

__all__ = ["kernels", "FastQSL"]

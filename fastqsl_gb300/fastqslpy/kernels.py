"""Drop-in for fastqslpy/kernels.py.

``compileTraceBlineAdaptive()`` / ``compileTraceBlineRK4()`` return a callable
with ``cupy.RawKernel``'s call convention, ``k(grid, block, args)``, taking
the reference kernel's argument tuple (TraceBlineAdaptive.cu:429-437, 35
arguments; TraceBline.cu:383-391, 34 arguments; extra trailing arguments are
ignored as the RK4 kernel ignores the notebooks' trailing tol_coef).  Nothing
is compiled at run time: the kernels are the prebuilt sm_103a code of
libfastqsl_gb300.so.  `grid` and `block` are accepted and ignored; the launch
geometry is a persistent grid sized to the GPU.
"""
from .. import _lib
from ..api import ptr

RK4 = 0
RKF45 = 1
_ARITH = {"exact": 0, "fast": 1}


def _current_stream(args):
    for a in args:
        if hasattr(a, "__cuda_array_interface__") and not hasattr(a, "data_ptr"):
            try:
                import cupy  # the caller's arrays are CuPy: use CuPy's current stream
                return cupy.cuda.get_current_stream().ptr
            except ImportError:
                break
    import torch
    return torch.cuda.current_stream().cuda_stream


# argument positions of the per-seed arrays: inp_x/y/z (9-11), start ..
# B_end_z (13-30), LineLen (33)
_PER_SEED = [9, 10, 11] + list(range(13, 31)) + [33]


def _numel(a):
    if hasattr(a, "numel"):
        return int(a.numel())
    return int(getattr(a, "size", 0))


class TraceAllBline:
    """The reference's TraceAllBline kernel object."""

    def __init__(self, integrator, arith="exact"):
        if arith not in _ARITH:
            raise ValueError("arith must be 'exact' or 'fast'")
        self.integrator = integrator
        self.arith = arith
        self.nargs = 35 if integrator == RKF45 else 34
        _lib.load()

    def __call__(self, grid, block, args, shared_mem=0, stream=None):
        args = tuple(args)
        if len(args) < self.nargs:
            raise TypeError(f"TraceAllBline takes {self.nargs} arguments, got {len(args)}")
        # the per-seed arrays bound the number of lines the kernel may touch
        cap = min(_numel(args[i]) for i in _PER_SEED)
        p = [ptr(a) if _numel(a) else None for a in args[:self.nargs]]
        if self.integrator == RK4:
            p.append(None)  # no tol_coef
        st = stream if stream is not None else _current_stream(args)
        lib = _lib.load()
        _lib.check(lib.qsl_trace_all_bline(self.integrator, _ARITH[self.arith], *p, cap, st), "TraceAllBline")


class TraceAllBlineScott:
    """The Scott kernel TraceAllBlineScott (TraceBlineScott.cu:521-528, 30
    arguments), which the reference's Scott notebooks compile themselves;
    exact arithmetic, central-difference gradient."""

    # inp_x/y/z (9-11), start..q_perp (13-25), LineLen (28)
    _PER_SEED = [9, 10, 11] + list(range(13, 26)) + [28]

    def __init__(self):
        _lib.load()

    def __call__(self, grid, block, args, shared_mem=0, stream=None):
        args = tuple(args)
        if len(args) < 30:
            raise TypeError(f"TraceAllBlineScott takes 30 arguments, got {len(args)}")
        cap = min(_numel(args[i]) for i in self._PER_SEED)
        p = [ptr(a) if _numel(a) else None for a in args[:30]]
        st = stream if stream is not None else _current_stream(args)
        _lib.check(_lib.load().qsl_trace_all_bline_scott(*p, cap, st), "TraceAllBlineScott")


class TraceAllBlineStretch:
    """TraceAllBline of fastqslpy/cu/TraceBlineAdaptiveStretch.cu:422-433 (39
    arguments: the field, BshapeN, x_arr, y_arr, z_arr, flag_uni, then the
    35-argument list of the uniform-grid kernel from curB_x on), which the
    reference's stretched-grid notebook compiles itself."""

    # inp_x/y/z (13-15), start..B_end_z (17-34), LineLen (37)
    _PER_SEED = [13, 14, 15] + list(range(17, 35)) + [37]

    def __init__(self, arith="exact"):
        if arith not in _ARITH:
            raise ValueError("arith must be 'exact' or 'fast'")
        self.arith = arith
        _lib.load()

    def __call__(self, grid, block, args, shared_mem=0, stream=None):
        args = tuple(args)
        if len(args) < 39:
            raise TypeError(f"TraceAllBline (stretched grid) takes 39 arguments, got {len(args)}")
        cap = min(_numel(args[i]) for i in self._PER_SEED)
        p = [ptr(a) if _numel(a) else None for a in args[:39]]
        st = stream if stream is not None else _current_stream(args)
        _lib.check(_lib.load().qsl_trace_all_bline_stretch(_ARITH[self.arith], *p, cap, st),
                   "TraceAllBline (stretched grid)")


def compileTraceBlineAdaptiveStretch(arith="exact"):
    """RKF45 tracer on a stretched grid (the reference's stretched notebook
    compiles fastqslpy/cu/TraceBlineAdaptiveStretch.cu and takes TraceAllBline)."""
    return TraceAllBlineStretch(arith)


def compileTraceBlineScott():
    """Scott deviation-vector tracer (reference notebooks compile
    fastqslpy/cu/TraceBlineScott.cu and take TraceAllBlineScott)."""
    return TraceAllBlineScott()


def compileTraceBlineAdaptive(arith="exact"):
    """RKF45 tracer (reference: fastqslpy/kernels.py:10-18)."""
    return TraceAllBline(RKF45, arith)


def compileTraceBlineRK4(arith="exact"):
    """Fixed-step RK4 tracer (reference: fastqslpy/kernels.py:21-29)."""
    return TraceAllBline(RK4, arith)

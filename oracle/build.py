"""Builds the CPU oracle (test infrastructure).

* ``oracle/_build/libqsl_oracle.so`` — the C restatement in oracle/port
  (FP32 reference-parity ``qo32_*``, the same with a correctly rounded
  power ``qo32cr_*``, and FP64 ``qo64_*``), OpenMP-parallel.
  Built on every machine (it is the checker on the GPU host as well).
* ``oracle/_ref/libqslref_{rk4,rkf45,scott,stretch}.so`` — the reference's own kernels
  compiled for the host by ``oracle/build_ref.sh``; only where the reference
  checkout exists.

Both use -ffp-contract=off so float expressions round exactly as written on
x86-64 and on aarch64 alike.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
PORT_SO = os.path.join(BUILD, "libqsl_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
# the reference checkout: $QSL_REFERENCE_ROOT, else a directory named
# `reference` beside this repository
REFERENCE_ROOT = os.environ.get("QSL_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference"))

# -fno-strict-aliasing: on aarch64, GCC 13 at -O2 produced wrong stretched-
# grid samples of the port (differing from -O0, -O1 and every x86 build;
# AddressSanitizer and UBSan report nothing); without type-based alias
# analysis all builds agree bit for bit.
_CFLAGS = ["-O2", "-fno-strict-aliasing", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fvisibility=hidden", "-std=c11", "-I", os.path.join(ROOT, "include")]


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_port(force=False):
    src = os.path.join(HERE, "port", "qsl_port.c")
    hdr = os.path.join(ROOT, "include", "fastqsl_gb300.h")
    if not force and _newer(PORT_SO, [src, hdr, __file__]):
        return PORT_SO
    os.makedirs(BUILD, exist_ok=True)
    variants = [("qsl_port32.o", ["-DQO_REAL=float", "-DQO_DOUBLE=0", "-DQO_CRPOW=0"]),
                ("qsl_port32cr.o", ["-DQO_REAL=float", "-DQO_DOUBLE=0", "-DQO_CRPOW=1"]),
                ("qsl_port64.o", ["-DQO_REAL=double", "-DQO_DOUBLE=1", "-DQO_CRPOW=0"])]
    objs = [os.path.join(BUILD, o) for o, _ in variants]
    procs = [subprocess.Popen(["gcc", *_CFLAGS, *d, "-c", src, "-o", o]) for o, (_, d) in zip(objs, variants)]
    if any(p.wait() != 0 for p in procs):
        raise RuntimeError("oracle port compile failed")
    tmp = PORT_SO + ".tmp"
    subprocess.check_call(["gcc", "-shared", "-fopenmp", *objs, "-o", tmp, "-lm"])
    os.replace(tmp, PORT_SO)
    return PORT_SO


def reference_available(root=REFERENCE_ROOT):
    return os.path.isfile(os.path.join(root, "fastqslpy", "cu", "TraceBlineAdaptive.cu"))


def build_ref(root=REFERENCE_ROOT, force=False):
    """Compiles the reference kernels for the host; returns False when the
    reference checkout is absent."""
    if not reference_available(root):
        return False
    outs = [os.path.join(REF_DIR, f"libqslref_{k}.so") for k in ("rk4", "rkf45", "scott", "stretch")]
    srcs = [os.path.join(HERE, "ref_shim", f) for f in ("ref_driver.cpp", "cuda_runtime.h", "exports.map")]
    srcs.append(os.path.join(HERE, "build_ref.sh"))
    if not force and all(_newer(o, srcs) for o in outs):
        return True
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh"), root])
    return True


def build_all():
    build_port()
    build_ref()


if __name__ == "__main__":
    build_port(force="--force" in sys.argv)
    print("port:", PORT_SO)
    print("reference:", build_ref(force="--force" in sys.argv))

"""Builds the TensorFlow custom-op shim (tfq_gb300_tf_ops.cc) where
TensorFlow is installed:

    python -m quantum_gb300.tf_shim.build

compiles it with TensorFlow's own compile and link flags
(tf.sysconfig.get_compile_flags / get_link_flags) against
quantum_gb300/_lib/libtfq_gb300.so into
quantum_gb300/tf_shim/_tfq_gb300_tf_ops.so, which
tf.load_op_library() loads in place of the reference's op libraries.

syntax_check() compiles the same file against the stand-in headers in stub/
(no TensorFlow needed), which keeps it in step with include/tfq_gb300.h."""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
SRC = os.path.join(HERE, "tfq_gb300_tf_ops.cc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
OUT = os.path.join(HERE, "_tfq_gb300_tf_ops.so")


def syntax_check():
    """g++ -fsyntax-only against the stand-in TensorFlow headers; returns
    the compiler output, raises on an error."""
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(HERE, "stub"),
           "-I", INCLUDE, SRC]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("tf shim syntax check failed:\n" + r.stdout)
    return r.stdout


def build():
    """Compile the shim against the installed TensorFlow; returns the .so
    path.  Raises ImportError where TensorFlow is absent."""
    import tensorflow as tf  # noqa: F401  (only where TensorFlow is installed)
    from quantum_gb300 import build as native_build
    lib = native_build.build()
    cflags = tf.sysconfig.get_compile_flags()
    lflags = tf.sysconfig.get_link_flags()
    cmd = (["g++", "-std=c++17", "-O2", "-shared", "-fPIC", SRC, "-o", OUT, "-I", INCLUDE]
           + cflags + lflags + [lib, "-Wl,-rpath," + os.path.dirname(lib)])
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("tf shim build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return OUT


def load():
    """tf.load_op_library of the built shim (builds it first if needed)."""
    import tensorflow as tf
    if not os.path.exists(OUT):
        build()
    return tf.load_op_library(OUT)


if __name__ == "__main__":
    try:
        print(build())
    except ImportError:
        print("TensorFlow is not installed here: shim not built; syntax check:",
              syntax_check() or "ok")
        sys.exit(0)

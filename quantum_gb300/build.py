"""In-tree build of the native library (no cmake, no setuptools).

    python -m quantum_gb300.build

compiles quantum_gb300/csrc into quantum_gb300/_lib/libtfq_gb300.so for
sm_103a: host C++ with g++, kernels with nvcc, translation units in
parallel, rebuilt only when a source is newer than the library.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_NAME = "libtfq_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("CUDA toolkit not found (set CUDA_HOME)")


def lib_path():
    return os.path.join(OUT_DIR, LIB_NAME)


def _sources():
    names = sorted(os.listdir(CSRC))
    srcs = [os.path.join(CSRC, n) for n in names if n.endswith((".cc", ".cu"))]
    deps = [os.path.join(CSRC, n) for n in names
            if n.endswith((".h", ".cuh", ".cc", ".cu"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "tfq_gb300.h"))
    return srcs, deps


JIT_HEADERS = ("sim_device.cuh", "kernels.h", "tfqg_types.h", "rtc_types.h")


def _write_jit_headers(obj_dir):
    """Embed the device headers the run-time compiler needs."""
    out = os.path.join(obj_dir, "jit_headers.cc")
    parts = ["// generated by quantum_gb300/build.py: device headers for NVRTC",
             "namespace tfqg {"]
    names, srcs = [], []
    for h in JIT_HEADERS:
        text = open(os.path.join(CSRC, h)).read()
        assert ")TFQGJIT\"" not in text
        names.append(f'"{h}"')
        srcs.append('R"TFQGJIT(' + text + ')TFQGJIT"')
    parts.append("extern const char* const kJitHeaderNames[] = {" + ", ".join(names) + "};")
    parts.append("extern const char* const kJitHeaderSources[] = {\n" + ",\n".join(srcs) + "};")
    parts.append(f"extern const int kJitHeaderCount = {len(JIT_HEADERS)};")
    parts.append("}  // namespace tfqg")
    text = "\n".join(parts) + "\n"
    if not os.path.exists(out) or open(out).read() != text:
        with open(out, "w") as f:
            f.write(text)
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _depfile_deps(dep):
    """Files listed in a make-style dependency file (None if unreadable)."""
    try:
        text = open(dep).read()
    except OSError:
        return None
    text = text.replace("\\\n", " ")
    _, _, rest = text.partition(":")
    return [t for t in rest.split() if t]


def _obj_stale(obj, src):
    if not os.path.exists(obj):
        return True
    deps = _depfile_deps(obj + ".d")
    if deps is None:
        return True
    return _stale(obj, [src, os.path.abspath(__file__)] + deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force=False, verbose=False):
    """Compile the library if needed; return its path."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    srcs, deps = _sources()
    out = lib_path()
    if not force and not _stale(out, deps):
        return out
    os.makedirs(OUT_DIR, exist_ok=True)
    obj_dir = os.path.join(OUT_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    inc = ["-I" + CSRC, "-I" + os.path.join(cuda, "include")]
    cmds = []
    objs = []
    srcs = srcs + [_write_jit_headers(obj_dir)]
    cuda_lib = os.path.join(cuda, "lib64")
    for src in srcs:
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if not force and not _obj_stale(obj, src):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17",
                                   "-Xcompiler", "-fPIC", "-Xptxas", "-v",
                                   "-MD", "-MF", obj + ".d",
                                   "-c", src, "-o", obj] + inc
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-pthread",
                   f'-DTFQG_CUDA_LIB_DIR="{cuda_lib}"', "-MMD", "-MF", obj + ".d",
                   "-c", src, "-o", obj] + inc
        cmds.append(cmd)
    if cmds:
        with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
            logs = list(ex.map(_run, cmds))
        if verbose:
            for log in logs:
                sys.stdout.write(log)
    tmp = out + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs +
         ["-L" + cuda_lib, "-ldl", "-lpthread"])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)

"""Build the native library ``libpdq_gb300.so`` in-tree for sm_103a.

Each ``csrc/*.cu`` translation unit compiles in its own ``nvcc`` process (in
parallel), then one shared object is linked with the CUDA runtime statically
linked in.  Outputs: ``probdiffeq_gb300/libpdq_gb300.so`` (object files go to
``_build/`` at the repository root).
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libpdq_gb300.so")

GENCODE = "arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    "-gencode",
    GENCODE,
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-I" + INCLUDE,
    "-I" + CSRC,
    "-I" + BUILD,
]

# Headers compiled at run time (NVRTC) together with user vector fields; they
# are embedded in the library as string literals.
EMBEDDED_HEADERS = [
    ("pdq.h", os.path.join(INCLUDE, "pdq.h")),
    ("pdq_device.cuh", os.path.join(CSRC, "pdq_device.cuh")),
    ("iso_solver.cuh", os.path.join(CSRC, "iso_solver.cuh")),
    ("iso_lean.cuh", os.path.join(CSRC, "iso_lean.cuh")),
    ("dense_solver.cuh", os.path.join(CSRC, "dense_solver.cuh")),
    ("lml_solver.cuh", os.path.join(CSRC, "lml_solver.cuh")),
    ("lml_adjoint.cuh", os.path.join(CSRC, "lml_adjoint.cuh")),
    ("bd_solver.cuh", os.path.join(CSRC, "bd_solver.cuh")),
]


def write_embedded_headers():
    """Generate ``_build/pdq_embedded_headers.inc`` (raw string literals of the headers)."""
    os.makedirs(BUILD, exist_ok=True)
    names, bodies = [], []
    for name, path in EMBEDDED_HEADERS:
        with open(path) as f:
            text = f.read()
        delim = "PDQHDR"
        if ")" + delim + '"' in text:
            raise RuntimeError(f"{name} contains the raw-string delimiter")
        names.append('"' + name + '"')
        bodies.append('R"' + delim + "(" + text + ")" + delim + '"')
    out = "// generated by probdiffeq_gb300/build.py from the solver headers\n"
    out += f"static const int kPdqHeaderCount = {len(names)};\n"
    out += "static const char* const kPdqHeaderNames[] = {" + ", ".join(names) + "};\n"
    out += "static const char* const kPdqHeaderSources[] = {\n" + ",\n".join(bodies) + "};\n"
    path = os.path.join(BUILD, "pdq_embedded_headers.inc")
    old = open(path).read() if os.path.exists(path) else None
    if old != out:
        with open(path, "w") as f:
            f.write(out)


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the native library cannot be built")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _newest_input_mtime():
    files = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def is_stale():
    return not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest_input_mtime()


def build(force=False, verbose=False):
    """Compile every translation unit and link the shared library."""
    if not force and not is_stale():
        return LIB
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    write_embedded_headers()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, *NVCC_FLAGS, "-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
        if verbose:
            sys.stdout.write(res.stdout + res.stderr)
        return obj

    srcs = sources()
    workers = min(len(srcs), max(1, os.cpu_count() or 1))
    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-gencode", GENCODE, "-shared", "-o", tmp, *objs, "-lnvrtc"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


JAX_FFI_SRC = os.path.join(PKG, "jax_ffi", "ffi_pdq.cc")
JAX_FFI_LIB = os.path.join(PKG, "libpdq_jax_ffi.so")


def jax_ffi_include_dir():
    """The directory holding jaxlib's xla/ffi/api/ffi.h, or None when jaxlib is not installed."""
    try:
        import jax.ffi

        cands = [jax.ffi.include_dir()]
    except Exception:  # no jax, or a jax without ffi.include_dir
        cands = []
    try:
        import jaxlib

        cands.append(os.path.join(os.path.dirname(jaxlib.__file__), "include"))
    except Exception:
        pass
    for d in cands:
        if os.path.exists(os.path.join(d, "xla", "ffi", "api", "ffi.h")):
            return d
    return None


def build_jax_ffi(force=False):
    """Compile the XLA FFI handlers (jax_ffi/ffi_pdq.cc) against jaxlib's
    headers into libpdq_jax_ffi.so, linked to libpdq_gb300.so; returns its
    path, or None (nothing built) when jaxlib's headers are not found."""
    inc = jax_ffi_include_dir()
    if inc is None:
        return None
    lib = build()
    if not force and os.path.exists(JAX_FFI_LIB) and os.path.getmtime(JAX_FFI_LIB) >= max(
            os.path.getmtime(JAX_FFI_SRC), os.path.getmtime(lib)):
        return JAX_FFI_LIB
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc_path())), "include")
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-I" + inc, "-I" + INCLUDE,
           "-I" + cuda_inc, JAX_FFI_SRC, "-o", JAX_FFI_LIB, "-L" + PKG, "-lpdq_gb300", "-Wl,-rpath,$ORIGIN"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"jax ffi build failed:\n{res.stdout}\n{res.stderr}")
    return JAX_FFI_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_jax_ffi(force="--force" in sys.argv) or "jax ffi handlers: jaxlib headers not found, not built")

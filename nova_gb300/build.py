"""Build recipe for libnova.so, the nova-gb300 C-ABI library.

Every translation unit is compiled by nvcc for sm_103a only (one -gencode),
in parallel, into nova_gb300/_build/, and linked into nova_gb300/lib/libnova.so
with the CUDA runtime linked statically. Host code is compiled without FMA
contraction so that host-side arithmetic matches on x86 and Arm.

Usage:  python -m nova_gb300.build   (or nova_gb300.build.build())
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib", "libnova.so")

SOURCES = ["runtime.cpp", "mdp_vi.cu", "mdp_vi_tiled.cu", "pbvi.cu", "pbvi_tc.cu", "pbvi_adjoint.cu", "pbvi_batched.cu", "expand.cu", "value_batched.cu", "loaders.cpp", "perseus.cu", "value_noalloc.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "--default-stream", "per-thread", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def exported_symbols():
    """Entry points declared with NOVA_API in include/nova/**/*.h (the C ABI)."""
    import re
    names = []
    for dirpath, _, files in os.walk(os.path.join(ROOT, "include")):
        for f in sorted(files):
            if f.endswith(".h"):
                text = "\n".join(l for l in open(os.path.join(dirpath, f)).read().split("\n")
                                 if not l.lstrip().startswith("#"))
                for m in re.finditer(r"NOVA_API\s+[\w\s\*]+?\b(\w+)\s*\(", text):
                    if m.group(1) not in names:
                        names.append(m.group(1))
    return names


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _header_mtimes():
    out = []
    for base in (CSRC, os.path.join(ROOT, "include")):
        for dirpath, _, files in os.walk(base):
            out += [os.path.getmtime(os.path.join(dirpath, f)) for f in files if f.endswith(".h")]
    return out


def _flags_stamp():
    """Objects are rebuilt when the compiler flags change, not only when sources do."""
    stamp = os.path.join(BUILD, "flags.txt")
    flags = " ".join(ARCH + COMMON)
    old = open(stamp).read() if os.path.exists(stamp) else None
    if old != flags:
        with open(stamp, "w") as f:
            f.write(flags)
    return os.path.getmtime(stamp)


def _compile(src, verbose, stamp_mtime=0.0):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max([os.path.getmtime(srcp), stamp_mtime] +
                                                            _header_mtimes()):
        return obj
    cmd = [_nvcc(), "-c", srcp, "-o", obj] + ARCH + COMMON
    if src.endswith(".cpp"):
        cmd = [_nvcc(), "-x", "cu", "-c", srcp, "-o", obj] + ARCH + COMMON
    if verbose:
        cmd.append("-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), res.stderr))
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def build(verbose=False):
    """Compile every CUDA/C++ source for sm_103a and link lib/libnova.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    stamp_mtime = _flags_stamp()
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, stamp_mtime), SOURCES))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + ".tmp"
    # Export exactly the C ABI declared in include/; everything else stays local.
    vscript = os.path.join(BUILD, "exports.map")
    with open(vscript, "w") as f:
        f.write("{\n  global:\n" + "".join("    %s;\n" % n for n in exported_symbols()) + "  local: *;\n};\n")
    cmd = [_nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC,-pthread", "-cudart", "static",
                                                          "-Xlinker", "--version-script=" + vscript]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), res.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

"""In-tree build of the engine library (and of the CPU oracle used by the tests).

Outputs (git-ignored, rebuilt on every machine; nothing compiled elsewhere is
reused):
  qpc-tdse-cpc_gb300/libqpc_gb300.so   engine: CUDA kernels for sm_103a + host setup
  oracle/_build/liboracle_cn.so        CPU oracle (test infrastructure only)
"""
import os
import platform
import subprocess
import sys
import concurrent.futures as cf

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "libqpc_gb300.so")
OBJDIR = os.path.join(PKG, "_build")
ORACLE_SRCS = [os.path.join(ROOT, "oracle", f) for f in ("oracle_cn.cpp", "oracle_arnoldi.cpp")]
ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "liboracle_cn.so")

NVCC_ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build_engine(force=False, verbose=False):
    srcs = [os.path.join(CSRC, f) for f in ("qpc_engine.cu", "qpc_setup.cpp", "qpc_internal.h", "qpc_chain.cuh",
                                             "qpc_noalloc.cu", "qpc_spectra.cpp", "qpc_arnoldi.cu", "qpc_cuda_util.cuh",
                                             "qpc_mlp.cu", "qpc_vgwr.cu", "qpc_momentum.cu", "qpc_momentum.cpp",
                                             "qpc_gemm.cuh", "qpc_hhg.cu", "qpc_ozaki.cu", "qpc_ozaki.cuh",
                                             "qpc_tcgen05.cuh", "qpc_ltrans.cu", "qpc_ltrans.cuh")]
    srcs.append(os.path.join(ROOT, "include", "qpc_gb300.h"))
    if not force and not _stale(LIB, srcs):
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    o_cu = os.path.join(OBJDIR, "qpc_engine.o")
    o_na = os.path.join(OBJDIR, "qpc_noalloc.o")
    o_cc = os.path.join(OBJDIR, "qpc_setup.o")
    o_sp = os.path.join(OBJDIR, "qpc_spectra.o")
    o_ar = os.path.join(OBJDIR, "qpc_arnoldi.o")
    o_ml = os.path.join(OBJDIR, "qpc_mlp.o")
    o_vg = os.path.join(OBJDIR, "qpc_vgwr.o")
    o_mo = os.path.join(OBJDIR, "qpc_momentum_cu.o")
    o_mt = os.path.join(OBJDIR, "qpc_momentum.o")
    o_hh = os.path.join(OBJDIR, "qpc_hhg.o")
    o_oz = os.path.join(OBJDIR, "qpc_ozaki.o")
    o_lt = os.path.join(OBJDIR, "qpc_ltrans.o")
    nv = [_nvcc()] + NVCC_ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"] + os.environ.get("QPC_NVCC_EXTRA", "").split()
    jobs = [
        nv + ["-c", os.path.join(CSRC, "qpc_engine.cu"), "-o", o_cu],
        nv + ["-c", os.path.join(CSRC, "qpc_noalloc.cu"), "-o", o_na],
        nv + ["-c", os.path.join(CSRC, "qpc_arnoldi.cu"), "-o", o_ar],
        nv + ["-c", os.path.join(CSRC, "qpc_mlp.cu"), "-o", o_ml],
        nv + ["-c", os.path.join(CSRC, "qpc_vgwr.cu"), "-o", o_vg],
        nv + ["-c", os.path.join(CSRC, "qpc_momentum.cu"), "-o", o_mo],
        nv + ["-c", os.path.join(CSRC, "qpc_hhg.cu"), "-o", o_hh],
        nv + ["-c", os.path.join(CSRC, "qpc_ozaki.cu"), "-o", o_oz],
        nv + ["-c", os.path.join(CSRC, "qpc_ltrans.cu"), "-o", o_lt],
        ["g++", "-O2", "-std=c++17", "-fPIC", "-c", os.path.join(CSRC, "qpc_momentum.cpp"), "-o", o_mt],
        ["g++", "-O2", "-std=c++17", "-fPIC", "-c", os.path.join(CSRC, "qpc_setup.cpp"), "-o", o_cc],
        ["g++", "-O2", "-std=c++17", "-fPIC", "-c", os.path.join(CSRC, "qpc_spectra.cpp"), "-o", o_sp],
    ]
    with cf.ThreadPoolExecutor(len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    _run([_nvcc()] + NVCC_ARCH + ["-shared", o_cu, o_na, o_ar, o_ml, o_vg, o_mo, o_hh, o_oz, o_lt, o_mt, o_cc, o_sp, "-o", LIB + ".tmp", "-lcudart", "-lcusolver", "-lpthread"])
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("".join(outs))
    return LIB


def build_oracle(force=False):
    if not force and not _stale(ORACLE_LIB, ORACLE_SRCS):
        return ORACLE_LIB
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    # fma() must be the hardware instruction (exactly rounded either way); on
    # x86-64 that needs -mfma, on aarch64 it is baseline
    isa = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
    _run(["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"] + isa +
         ORACLE_SRCS + ["-o", ORACLE_LIB + ".tmp"])
    os.replace(ORACLE_LIB + ".tmp", ORACLE_LIB)
    return ORACLE_LIB


def build_reference_oracle(ref_dir=None):
    """Build the reference's own propagator into oracle/_ref/ from the reference
    checkout (test infrastructure: the golden fixtures are made with it).  The
    checkout is ref_dir, else the environment variable QPC_REFERENCE_DIR, else the
    development machine's checkout location; nothing is built when none exists (a
    GPU machine has none)."""
    cands = [ref_dir, os.environ.get("QPC_REFERENCE_DIR"), "/root/reference"]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "include")):
            _run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), "-j4", "REF_INCLUDE=" + os.path.join(c, "include")])
            return os.path.join(ROOT, "oracle", "_ref")
    return None


if __name__ == "__main__":
    f = "--force" in sys.argv
    print(build_engine(f, verbose=True))
    print(build_oracle(f))

"""Build the gnuts shared library (CUDA, sm_103a) and the CPU oracle.

Compiles in-tree with nvcc / g++ directly (no cmake), in parallel, and only
what changed.  Outputs:
    cmdstan_gb300/_lib/libgnuts.so     the product (C ABI of include/gnuts.h)
    cmdstan_gb300/_lib/gnuts-sample    CmdStan-compatible command line
    cmdstan_gb300/_lib/gnuts-diagnose  the diagnose tool over Stan CSV files
    oracle/_build/liboracle.so         CPU oracle (test infrastructure)
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
CLI = os.path.join(HERE, "cli")
LIB = os.path.join(HERE, "_lib")
INC = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-I" + INC, "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I" + INC, "-I" + CSRC]

CU_SOURCES = ["sampler.cu", "fused.cu", "grad_tc.cu", "grad_wide.cu", "noalloc.cu", "flow.cu", "summary_gpu.cu"]
# compiled once per model kind (-DGNUTS_KIND=k, k = 0..N_KINDS-1)
CU_KIND_SOURCES = ["fused_kind.cu", "flow_tc_kind.cu"]
N_KINDS = 7
# compiled once per (metric, team width) of the round-mode state machine
ADVANCE_SOURCE = "advance_kind.cu"
ADVANCE_VARIANTS = [(m, tw) for tw in (32, 128) for m in (0, 1, 2)]
CPP_SOURCES = ["abi.cpp", "summary.cpp", "learned.cpp", "diagnose.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INC, "gnuts.h"))
    return hs


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(verbose=False, jobs=None):
    os.makedirs(LIB, exist_ok=True)
    objdir = os.path.join(LIB, "obj")
    os.makedirs(objdir, exist_ok=True)
    nvcc = _nvcc()
    cuda = _cuda_home()
    headers = _headers()
    cmds = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(objdir, src + ".o")
        objs.append(o)
        if _newer(o, [s] + headers):
            cmds.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    for src in CU_KIND_SOURCES:
        s = os.path.join(CSRC, src)
        for k in range(N_KINDS):
            o = os.path.join(objdir, "%s.k%d.o" % (src, k))
            objs.append(o)
            if _newer(o, [s] + headers):
                cmds.append([nvcc] + NVCC_FLAGS + ["-DGNUTS_KIND=%d" % k, "-c", s, "-o", o])
    s = os.path.join(CSRC, ADVANCE_SOURCE)
    for m, tw in ADVANCE_VARIANTS:
        o = os.path.join(objdir, "%s.m%d.t%d.o" % (ADVANCE_SOURCE, m, tw))
        objs.append(o)
        if _newer(o, [s] + headers):
            cmds.append([nvcc] + NVCC_FLAGS + ["-DGNUTS_MET=%d" % m, "-DGNUTS_TW=%d" % tw, "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(objdir, src + ".o")
        objs.append(o)
        if _newer(o, [s] + headers):
            cmds.append(["g++"] + CXX_FLAGS + ["-I" + os.path.join(cuda, "include"), "-c", s, "-o", o])
    # oracle (test infrastructure) builds alongside
    oracle_cmd = ["make", "-s", "-C", ORACLE]
    with cf.ThreadPoolExecutor(max_workers=jobs or min(os.cpu_count() or 8, len(cmds) + 1)) as ex:
        futs = [ex.submit(_run, c) for c in cmds] + [ex.submit(_run, oracle_cmd)]
        for f in futs:
            out = f.result()
            if verbose and out.strip():
                print(out)
    so = os.path.join(LIB, "libgnuts.so")
    if _newer(so, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", so] + objs + ["-lcudart"])
    cli_src = os.path.join(CLI, "gnuts_sample.cpp")
    exe = os.path.join(LIB, "gnuts-sample")
    cli_deps = [os.path.join(CLI, f) for f in os.listdir(CLI)] if os.path.isdir(CLI) else []
    if os.path.exists(cli_src) and _newer(exe, cli_deps + [so, os.path.join(INC, "gnuts.h")]):
        _run(["g++"] + CXX_FLAGS + ["-pthread", "-I" + CLI, cli_src, "-o", exe, "-L" + LIB, "-lgnuts",
                                    "-Wl,-rpath,$ORIGIN"])
    diag_src = os.path.join(CLI, "gnuts_diagnose.cpp")
    diag_exe = os.path.join(LIB, "gnuts-diagnose")
    if os.path.exists(diag_src) and _newer(diag_exe, [diag_src, so, os.path.join(INC, "gnuts.h")]):
        _run(["g++"] + CXX_FLAGS + [diag_src, "-o", diag_exe, "-L" + LIB, "-lgnuts", "-Wl,-rpath,$ORIGIN"])
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

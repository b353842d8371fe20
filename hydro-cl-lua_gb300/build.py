"""Builds libhydrocuda.so in place (sm_103a) from csrc/ with nvcc.

Translation units compile in parallel.  The files whose results must match
the reference's arithmetic bit for bit (the plain FP64 kernels and the FP64
fused kernels) are compiled with -fmad=false; the FP32 fused kernels use the
fast single-precision intrinsics.
"""
import concurrent.futures
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhydrocuda.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + CSRC, "-I" + INCLUDE,
          "--expt-relaxed-constexpr"]
EXACT = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"]
FAST = ["-use_fast_math", "-ftz=false"]

SOURCES = {
    "hc_api.cu": [],
    "hc_plan.cu": [],
    "hc_plain.cu": EXACT,
    "hc_init.cu": EXACT,
    "hc_viz.cu": EXACT,
    "hc_fused_host.cu": [],
    "hc_fused_f32_d1.cu": FAST,
    "hc_fused_f32_d2a.cu": FAST,
    "hc_fused_f32_d2b.cu": FAST,
    "hc_fused_f32_d2c.cu": FAST,
    "hc_fused_f32_d2d.cu": FAST,
    "hc_fused_f32_d2e.cu": FAST,
    "hc_fused_f32_flux.cu": FAST,
    "hc_fused_f32_recon.cu": FAST,
    "hc_fused_f32_d3.cu": FAST,
    "hc_fused_f32_d3b.cu": FAST,
    "hc_fused_f32_d3c.cu": FAST,
    "hc_fused_f32_m2.cu": FAST,
    "hc_fused_f32_m3.cu": FAST,
    "hc_fused_f32_m2b.cu": FAST,
    "hc_fused_f32_m2c.cu": FAST,
    "hc_probe.cu": [],
    "hc_fused_f64_d1.cu": EXACT,
    "hc_fused_f64_d2.cu": EXACT,
    "hc_fused_f64_d3.cu": EXACT,
}


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _digest(paths, flags):
    h = hashlib.sha1()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def _headers():
    hs = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "hydrocuda.h"))
    return hs


def _compile(src, flags, extra_verbose):
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    stamp = obj + ".sha1"
    allflags = ARCH + COMMON + flags + (["-Xptxas", "-v"] if extra_verbose else [])
    dig = _digest([os.path.join(CSRC, src)] + _headers(), allflags)
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == dig:
        return obj, ""
    cmd = [_nvcc()] + allflags + ["-c", os.path.join(CSRC, src), "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), p.stderr[-8000:]))
    with open(stamp, "w") as f:
        f.write(dig)
    return obj, p.stderr


def build(verbose=False, jobs=None):
    """Compile every translation unit and link libhydrocuda.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    objs = []
    logs = []
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {ex.submit(_compile, s, f, verbose): s for s, f in SOURCES.items()}
        for fut in concurrent.futures.as_completed(futs):
            obj, log = fut.result()
            objs.append(obj)
            if log:
                logs.append("== %s\n%s" % (futs[fut], log))
    objs.sort()
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        subprocess.check_call(cmd)
        os.replace(tmp, LIB)
    if verbose:
        sys.stderr.write("\n".join(logs))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)

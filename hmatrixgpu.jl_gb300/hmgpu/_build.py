"""Compiles libhmgpu.so for sm_103a with nvcc (in-tree, no install step)."""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libhmgpu.so")
REPO = os.path.dirname(PKG)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
          "--expt-relaxed-constexpr", "-I" + os.path.join(REPO, "include")]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


# Per-file flags: the assembly and tree kernels must not contract a*b+c into an
# FMA, so that matrix entries, ACA residuals and cluster centres round exactly
# as the reference's do.
PER_FILE = {"hm_build.cu": ["--fmad=false"], "hm_tree_dev.cu": ["--fmad=false"]}


def _compile(src, extra):
    obj = os.path.join(BUILD, src + ".o")
    cmd = [nvcc()] + ARCH + COMMON + PER_FILE.get(src, []) + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


# Headers the library compiles again at run time, with a user's entry function
# (NVRTC, hm_user.cpp): embedded in the library as strings.
EMBEDDED = (("hm_src_entry_cuh", "hm_entry.cuh"), ("hm_src_packjob_h", "hm_packjob.h"))


def _embedded_sources():
    """Writes _build/hm_sources.cpp, which defines each embedded header's text."""
    out = []
    for sym, name in EMBEDDED:
        with open(os.path.join(CSRC, name)) as f:
            text = f.read()
        if ')HMSRC"' in text:
            raise RuntimeError(f"{name} contains the raw-string delimiter")
        out.append(f'extern const char {sym}[];\nconst char {sym}[] = R"HMSRC({text})HMSRC";\n')
    path = os.path.join(BUILD, "hm_sources.cpp")
    with open(path, "w") as f:
        f.write("".join(out))
    return path


def build(verbose=False, extra=(), jobs=None):
    """Compile every source in csrc/ in parallel and link libhmgpu.so. Returns the path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sources() + [_embedded_sources()]
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err.strip():
                print(err)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, extra=["-Xptxas", "-v"] if "-v" in sys.argv else []))

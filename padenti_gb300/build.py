"""In-tree build of libpadenti_gb300.so (sm_103a).

Compiles padenti_gb300/csrc/*.cu with nvcc and *.cpp with g++, in parallel, into
padenti_gb300/_build/, and links the shared library.  Objects are rebuilt only
when a source or header is newer.  ``python -m padenti_gb300.build`` runs it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parent
REPO = ROOT.parent
CSRC = ROOT / "csrc"
OUT = ROOT / "_build"
LIB = OUT / "libpadenti_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _nvcc() -> str:
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found (CUDA toolkit required to build padenti_gb300)")
    return p


def _headers() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted((REPO / "include").glob("*.h"))


def _stale(obj: pathlib.Path, src: pathlib.Path, deps: list[pathlib.Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in [src, *deps])


# Headers compiled again at run time by NVRTC for user feature plugins; they are
# embedded into the library as raw string literals (_build/pd_rtc_sources.inc).
RTC_HEADERS = ["padenti_gb300.h", "pd_common.cuh", "pd_log2.cuh", "pd_rng.cuh", "pd_propose.cuh", "pd_plugins.cuh",
               "pd_train_kernels.cuh", "pd_predict_kernels.cuh", "pd_user_plugin.cuh", "pd_user_plugin_impl.cuh"]


def _embed_rtc_sources() -> None:
    out = OUT / "pd_rtc_sources.inc"
    parts = []
    for name in RTC_HEADERS:
        path = (REPO / "include" / name) if name.endswith(".h") else (CSRC / name)
        text = path.read_text()
        if ")pdrtc\"" in text:
            raise RuntimeError(f"{path} contains the raw-string delimiter")
        parts.append(f'{{"{name}", R"pdrtc({text})pdrtc"}},\n')
    data = "".join(parts)
    if not out.exists() or out.read_text() != data:
        out.write_text(data)


def _compile(src: pathlib.Path, extra: list[str]) -> pathlib.Path:
    obj = OUT / (src.name + ".o")
    inc = [f"-I{REPO / 'include'}", f"-I{CSRC}", f"-I{OUT}"]
    if src.suffix == ".cu":
        cmd = [_nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++20", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-ffp-contract=off", *inc, *extra, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-pthread", *inc,
               "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and os.environ.get("PD_BUILD_VERBOSE"):
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, extra_nvcc: list[str] | None = None) -> pathlib.Path:
    """Builds (if needed) and returns the path of libpadenti_gb300.so."""
    OUT.mkdir(parents=True, exist_ok=True)
    _embed_rtc_sources()
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    deps = _headers()
    todo = [s for s in srcs if force or _stale(OUT / (s.name + ".o"), s, deps)]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        list(ex.map(lambda s: _compile(s, extra_nvcc or []), todo))
    objs = [OUT / (s.name + ".o") for s in srcs]
    if force or todo or not LIB.exists():
        cmd = [_nvcc(), ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart", "-lnvrtc",
               "-Xlinker", f"-rpath,{CUDA_HOME}/lib64"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

"""The C-ABI library loads and exports every entry point include/padenti_gb300.h
declares; host-only entry points work without a GPU."""
import ctypes as C
import pathlib
import re

import numpy as np
import pytest

import padenti_gb300 as pg
from padenti_gb300 import _native as N

HEADER = pathlib.Path(__file__).resolve().parent.parent / "include" / "padenti_gb300.h"


def _declared():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(pd_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_bound_functions():
    assert set(_declared()) == set(N.EXPORTED)


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    for name in _declared():
        assert hasattr(lib, name), name
    assert lib.pd_version() >= 10000


def test_context_creation_reports_errors_without_crashing():
    cfg = pg.ForestConfig("depth_diff2", 3).c()
    h = C.c_void_p()
    bad = N.Config(99, 2, 1, 2, 4, 3)
    rc = N.lib().pd_ctx_create(C.byref(bad), 0, C.byref(h))
    assert rc == -4 and b"unknown plugin" in N.lib().pd_last_error()
    wrong = N.Config(1, 1, 1, 2, 4, 3)  # depth plugin with uint8 images
    assert N.lib().pd_ctx_create(C.byref(wrong), 0, C.byref(h)) == -1
    assert b"needs img_type" in N.lib().pd_last_error()
    # on a machine without a GPU a valid config fails with a CUDA error, not a crash
    rc = N.lib().pd_ctx_create(C.byref(cfg), 0, C.byref(h))
    if rc == 0:
        N.lib().pd_ctx_destroy(h)
    else:
        assert rc in (-1, -2)


def test_synth_is_deterministic_and_shaped():
    a = pg.synth_depth(7, 3, 64, 48, samples_per_image=100)
    b = pg.synth_depth(7, 3, 64, 48, samples_per_image=100)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    px, lb, sm = a
    assert px.min() >= 1 and lb.min() >= 1 and lb.max() <= 3
    assert np.all(np.diff(sm.astype(np.int64), axis=1) >= 0)
    # 10% of the samples on the background (label 1)
    bg = np.mean(lb.reshape(3, -1)[np.arange(3)[:, None], sm] == 1)
    assert 0.05 < bg < 0.2
    c = pg.synth_depth(7, 1, 64, 48, samples_per_image=100, first_image=2)
    assert np.array_equal(c[0][0], px[2])
    r = pg.synth_rgb(1, 2, 40, 30, n_classes=21, samples_per_image=50)
    assert r[0].shape == (2, 30, 40, 3) and r[1].max() <= 21


def test_python_api_fails_loudly_when_the_library_is_missing(monkeypatch, tmp_path):
    monkeypatch.setattr(N, "_lib", None)
    monkeypatch.setattr(N, "LIB_PATH", tmp_path / "missing.so")
    with pytest.raises(RuntimeError, match="missing"):
        N.lib()


def test_headers_compile_cleanly_as_c_and_cpp(tmp_path):
    """padenti_gb300.h is plain C (C99, pedantic); the C++ façade headers build without
    warnings under -Wall -Wextra -Wpedantic."""
    import shutil
    import subprocess

    inc = str(HEADER.parent)
    if shutil.which("gcc"):
        c = tmp_path / "h.c"
        c.write_text("#include <padenti_gb300.h>\nint main(void) { pd_sampler s; (void)s; return 0; }\n")
        r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Wpedantic", "-Werror", f"-I{inc}",
                            "-fsyntax-only", str(c)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    if shutil.which("g++"):
        cpp = tmp_path / "h.cpp"
        cpp.write_text("".join(f"#include <padenti/{h}>\n" for h in
                               ["cuda_tree_trainer.hpp", "image_sampler.hpp", "image_loader.hpp", "classifier.hpp",
                                "tree_trainer.hpp", "training_set.hpp", "tree.hpp", "image.hpp"]) + "int main() {}\n")
        r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Wpedantic", "-Werror", f"-I{inc}",
                            "-fsyntax-only", str(cpp)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def _compile_cpp(tmp_path, body: str, link: bool = False):
    import subprocess

    inc = str(HEADER.parent)
    src = tmp_path / "t.cpp"
    src.write_text("#include <padenti/cuda_tree_trainer.hpp>\n" + body)
    cmd = ["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", f"-I{inc}"]
    if link:
        lib = N.LIB_PATH
        cmd += [str(src), "-o", str(tmp_path / "t"), f"-L{lib.parent}", "-lpadenti_gb300",
                f"-Wl,-rpath,{lib.parent}"]
    else:
        cmd += ["-fsyntax-only", str(src)]
    return subprocess.run(cmd, capture_output=True, text=True)


def test_facade_refuses_types_without_kernels(tmp_path):
    """Image or feature types without kernels do not compile (the reference would throw at run
    time); the supported ones do."""
    import shutil

    if not shutil.which("g++"):
        pytest.skip("no g++")
    for img in ("unsigned short", "float", "short"):
        ok = _compile_cpp(tmp_path, f"void f() {{ CUDATreeTrainer<{img}, 1, int, 4, 3> t(1); (void)t; }}\n")
        assert ok.returncode == 0, ok.stderr
    for img, feat in (("double", "int"), ("unsigned short", "float"), ("unsigned short", "unsigned int")):
        r = _compile_cpp(tmp_path, f"void f() {{ CUDATreeTrainer<{img}, 1, {feat}, 4, 3> t(1); (void)t; }}\n")
        assert r.returncode != 0 and "padenti_gb300:" in r.stderr, (img, feat)


def test_facade_use_cpu_overload(tmp_path):
    """CUDATreeTrainer(path, bool useCPU) is the reference's constructor (cl_tree_trainer.hpp:115):
    useCPU=true is refused with an error (there is no CPU path), never read as device 1."""
    import shutil
    import subprocess

    if not shutil.which("g++"):
        pytest.skip("no g++")
    body = """#include <cstdio>
int main() {
  try {
    CUDATreeTrainer<unsigned short, 1, int, 4, 3> t(std::string("/nonexistent"), true);
    return 1;
  } catch (const std::exception &e) {
    std::puts(e.what());
  }
  try {
    CUDAClassifier<unsigned short, 1, int, 4, 3> c(std::string("/nonexistent"), true);
    return 1;
  } catch (const std::exception &e) {
    std::puts(e.what());
  }
  return 0;
}
"""
    r = _compile_cpp(tmp_path, body, link=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(tmp_path / "t")], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.count("useCPU=true") == 2, out.stdout + out.stderr

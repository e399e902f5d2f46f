"""INTEGRATION.md's reference-side adapters compile against the reference.

Every C++ block of INTEGRATION.md whose first line is a `// <path>.cpp`
comment is part of that file (blocks naming the same file are joined in
order). Each file is compiled with -fsyntax-only against include/mara_gb300.h,
the CUDA runtime headers and the reference's own src/ and problems/ headers,
with the reference's compile flags. Skipped where the reference checkout (the
oracle Makefile's REF) or the CUDA headers are absent.
"""
from __future__ import annotations

import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CUDA_INCLUDE = Path("/usr/local/cuda/include")


def reference_checkout() -> Path | None:
    res = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "print-ref"], capture_output=True, text=True)
    ref = Path(res.stdout.strip()) if res.returncode == 0 and res.stdout.strip() else None
    return ref if ref is not None and (ref / "problems" / "minidisk.hpp").exists() else None


def snippet_files() -> dict[str, str]:
    text = (ROOT / "INTEGRATION.md").read_text()
    files: dict[str, list[str]] = {}
    for block in re.findall(r"```cpp\n(.*?)```", text, flags=re.S):
        m = re.match(r"// (\S+\.cpp)\b", block)
        if m:
            files.setdefault(m.group(1), []).append(block)
    return {name: "\n".join(parts) for name, parts in files.items()}


def test_integration_has_compilable_snippets():
    files = snippet_files()
    assert {"problems/minidisk_gpu.cpp", "problems/minidisk_ensemble_gpu.cpp", "examples/mhd3d_gpu.cpp",
            "src/scheme_sedov2d_gpu.cpp", "problems/sedov2d_gpu.cpp"} <= set(files)
    assert "(continued)" in files["problems/minidisk_gpu.cpp"]


@pytest.mark.parametrize("name", sorted(snippet_files()))
def test_integration_snippet_compiles(name, tmp_path):
    ref = reference_checkout()
    if ref is None:
        pytest.skip("no reference checkout")
    if not CUDA_INCLUDE.exists() or shutil.which("g++") is None:
        pytest.skip("no CUDA headers or g++")
    src = tmp_path / Path(name).name
    src.write_text(snippet_files()[name])
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror=return-type", "-include", "stdexcept",
           "-include", "string", f"-I{ROOT / 'include'}", f"-I{CUDA_INCLUDE}", f"-I{ref / 'src'}",
           f"-I{ref / 'problems'}", str(src)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]

"""The static archive (lib/libsty_gb300.a) that a host links into its own binary: it defines every
entry point the header declares, and a C++ program linked against it (with the static CUDA runtime)
runs a host-only call with the same answer as the shared library. No GPU is used."""
import pathlib
import re
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "sty_gb300.h"
ARCHIVE = ROOT / "practical-stylized_gb300" / "lib" / "libsty_gb300.a"
CUDA = pathlib.Path("/usr/local/cuda")


def _declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"STY_API\s+[\w\s\*]+?\b(sty_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def archive(sty):
    if not ARCHIVE.exists():
        pytest.skip("static archive not built")
    return ARCHIVE


def test_archive_defines_every_entry_point(archive):
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-g", "--defined-only", str(archive)], capture_output=True, text=True, check=True).stdout
    defined = set(re.findall(r"\sT\s(sty_\w+)$", out, re.M))
    missing = [f for f in _declared() if f not in defined]
    assert not missing, missing
    assert len(_declared()) >= 40


def test_program_links_statically(archive, tmp_path, sty):
    gxx = shutil.which("g++")
    cudart = CUDA / "lib64" / "libcudart_static.a"
    if gxx is None or not cudart.exists():
        pytest.skip("g++ or the static CUDA runtime not available")
    src = tmp_path / "prog.cpp"
    src.write_text(
        '#include <cstdio>\n#include "sty_gb300.h"\n'
        'int main() { std::printf("%llu %llu\\n", (unsigned long long)sty_struct_size("sty_camera"),'
        ' (unsigned long long)sty_struct_size("sty_pf_records")); return 0; }\n')
    exe = tmp_path / "prog"
    subprocess.run([gxx, "-std=c++17", "-I", str(ROOT / "include"), str(src), str(archive), str(cudart),
                    "-lpthread", "-ldl", "-lrt", "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    lib = sty.abi.lib()
    assert int(out[0]) == lib.sty_struct_size(b"sty_camera")
    assert int(out[1]) == lib.sty_struct_size(b"sty_pf_records")
    assert int(out[0]) > 0

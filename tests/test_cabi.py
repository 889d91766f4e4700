"""The C-ABI library loads without a GPU and exports every entry point that
include/bgpu.h declares; the Python mirror binds all of them."""
import os
import re
import subprocess

from conftest import ROOT


def declared():
    with open(os.path.join(ROOT, "include", "bgpu.h")) as f:
        txt = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(bgpu_\w+)\s*\(", txt, flags=re.M)))


def test_library_exports_all_declarations():
    import block_gb300

    lib = block_gb300.load_library()
    names = declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", block_gb300.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if " T " in l)
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_python_mirror_covers_header():
    import block_gb300

    assert set(declared()) == set(block_gb300.EXPORTED)


def test_version_without_gpu():
    import block_gb300

    assert b"sm_103a" in block_gb300.load_library().bgpu_version()


def test_errors_without_gpu_are_reported():
    import block_gb300
    import torch

    if torch.cuda.is_available():
        return
    try:
        block_gb300.Context(0)
    except block_gb300.BgpuError as e:
        assert str(e)
    else:
        raise AssertionError("context creation must fail loudly without a GPU")


def test_plain_c_caller_builds_and_links(tmp_path):
    """include/bgpu.h is valid C: a C program that includes it, links the
    library and calls an entry point that needs no GPU."""
    import shutil

    import block_gb300

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        import pytest

        pytest.skip("no C compiler")
    src = tmp_path / "caller.c"
    src.write_text(
        '#include <stdio.h>\n#include "bgpu.h"\n'
        "int main(void) {\n"
        "  bgpu_ctx* ctx = 0;\n"
        "  const char* v = bgpu_version();\n"
        "  (void)ctx;\n"
        '  printf("%s\\n", v);\n'
        "  return v ? 0 : 1;\n}\n")
    exe = tmp_path / "caller"
    libdir = os.path.dirname(block_gb300.LIB_PATH)
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", str(src), "-I", os.path.join(ROOT, "include"), "-L", libdir,
                    "-lblockgb300", "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    assert "sm_103a" in out


def test_noalloc_limit_matches_header():
    import block_gb300

    with open(os.path.join(ROOT, "include", "bgpu.h")) as f:
        m = re.search(r"#define\s+BGPU_NOALLOC_SCRATCH_DOUBLES\s+\((\d+)\s*\*\s*(\d+)\s*\*\s*(\d+)\)", f.read())
    assert m, "BGPU_NOALLOC_SCRATCH_DOUBLES not found"
    assert int(m.group(1)) * int(m.group(2)) * int(m.group(3)) == block_gb300.NOALLOC_SCRATCH_DOUBLES

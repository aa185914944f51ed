"""The reference-side binding (include/wk_rcache_binding.hpp) compiles against
the reference's own request_or_reply (core/query.hpp:45-175) and config
globals, links libwkgpu.so, and maps each op's status to an exception.

Needs the reference headers that the oracle's `ref` target links into
oracle/_ref/src; skipped where they are absent (as on a machine without the
reference checkout)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_binding_compiles_against_request_or_reply(lib_built, tmp_path):
    src = ROOT / "oracle" / "_ref" / "src"
    if not (src / "query.hpp").exists() or shutil.which("g++") is None:
        pytest.skip("reference headers not linked (oracle ref target) or no g++")
    shim = ROOT / "oracle" / "ref_shim"
    exe = tmp_path / "rcache_binding_check"
    cmd = ["g++", "-O0", "-std=c++14", "-w", "-fpermissive", "-pthread", "-fopenmp",
           "-include", str(shim / "spin_hint.h")]
    for h in ("cstring", "map", "memory", "sstream", "unordered_map"):
        cmd += ["-include", h]
    cmd += [f"-I{src}", f"-I{shim}", f"-I{ROOT / 'include'}", "-o", str(exe),
            str(ROOT / "tests" / "binding" / "rcache_binding_check.cpp"),
            f"-L{ROOT / 'wukonggpu_gb300'}", "-lwkgpu", f"-Wl,-rpath,{ROOT / 'wukonggpu_gb300'}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    for op in ("known_to_unknown", "known_to_known", "known_to_const", "index_to_unknown"):
        assert f"{op} threw: device error" in r.stdout, r.stdout
    assert "binding check done" in r.stdout

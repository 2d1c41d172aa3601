"""The public C header and libvkhel.so as a C program sees them.

tests/c/test_vkhel_api.c includes only include/vkhel/vkhel.h and replays the
reference's golden operations with the reference test program's call
pattern.  On a CPU-only machine it must compile, link against libvkhel.so and
report the missing device cleanly (exit 77); on the GPU every case must match.
"""
import os
import subprocess

import pytest

from conftest import ROOT, load_golden

SRC = os.path.join(ROOT, "tests", "c", "test_vkhel_api.c")


def _build(tmp_path):
    from vkhel_gb300 import LIB_PATH
    exe = str(tmp_path / "test_vkhel_api")
    libdir = os.path.dirname(LIB_PATH)
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include", "vkhel"),
                    SRC, "-o", exe, "-L", libdir, "-lvkhel", f"-Wl,-rpath,{libdir}"], check=True)
    cases = tmp_path / "cases.txt"
    lines = []
    for op in load_golden("reference_vectors.json")["ops"]:
        p = op["params"]
        name = op["op"]
        if name in ("forward_transform", "inverse_transform"):
            params = [p["n"], p["q"], p["w"]]
        elif name == "elemfma":
            params = [p["multiplier"], p["mod"], "0"]
        elif name == "elemmul":
            params = [p["mod"], "0", "0"]
        elif name == "elemmod":
            params = [p["mod"], p["q"], "0"]
        elif name == "elemgtadd":
            params = [p["bound"], p["diff"], "0"]
        elif name == "elemgtsub":
            params = [p["bound"], p["diff"], p["mod"]]
        else:
            params = ["0", "0", "0"]
        lines.append(" ".join([name] + params))
        lines.append(" ".join(["a", str(len(op["a"]))] + op["a"]))
        if "b" in op:
            lines.append(" ".join(["b", str(len(op["b"]))] + op["b"]))
        lines.append(" ".join(["e", str(len(op["expected"]))] + op["expected"]))
    cases.write_text("\n".join(lines) + "\n")
    return exe, str(cases)


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_c_program_links_and_reports_no_device(vk, tmp_path):
    exe, cases = _build(tmp_path)
    r = subprocess.run([exe, cases], capture_output=True, text=True)
    assert r.returncode == 77 and "no CUDA device" in r.stdout


@pytest.mark.gpu
def test_c_program_replays_reference_golden_vectors(vk, tmp_path):
    exe, cases = _build(tmp_path)
    r = subprocess.run([exe, cases], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "35 cases, 0 failed" in r.stdout


EXT_SRC = os.path.join(ROOT, "tests", "c", "test_vkhel_ext.c")


def _build_ext(tmp_path):
    from vkhel_gb300 import LIB_PATH
    exe = str(tmp_path / "test_vkhel_ext")
    libdir = os.path.dirname(LIB_PATH)
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include", "vkhel"),
                    EXT_SRC, "-o", exe, "-L", libdir, "-lvkhel", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def _ext_args(n=1024):
    from vkhel_gb300 import workloads
    qs = workloads.ntt_primes(n, 3)
    return [str(n)] + [str(x) for q in qs for x in (q, workloads.root_for(n, q))]


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_c_extension_program_links_and_reports_no_device(vk, tmp_path):
    r = subprocess.run([_build_ext(tmp_path)] + _ext_args(), capture_output=True, text=True)
    assert r.returncode == 77 and "no CUDA device" in r.stdout


@pytest.mark.gpu
def test_c_extension_program_checks_pass(vk, tmp_path):
    r = subprocess.run([_build_ext(tmp_path)] + _ext_args(), capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 checks failed" in r.stdout


LAT_SRC = os.path.join(ROOT, "tests", "c", "call_latency.c")


def _latency_args():
    from vkhel_gb300 import workloads
    out = []
    for n in (16384, 4096, 65536):
        q = workloads.ntt_primes(n, 1)[0]
        out += [str(q), str(workloads.root_for(n, q))]
    return out


def _build_latency(tmp_path):
    from vkhel_gb300 import LIB_PATH
    exe = str(tmp_path / "call_latency")
    libdir = os.path.dirname(LIB_PATH)
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include", "vkhel"),
                    LAT_SRC, "-o", exe, "-L", libdir, "-lvkhel", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_call_latency_program_links_and_reports_no_device(vk, tmp_path):
    r = subprocess.run([_build_latency(tmp_path)] + _latency_args(), capture_output=True, text=True)
    assert r.returncode == 77


@pytest.mark.gpu
def test_call_latency_program_reports_every_call(vk, tmp_path):
    import json
    r = subprocess.run([_build_latency(tmp_path)] + _latency_args() + ["20"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    d = json.loads(r.stdout)
    for mode in ("blocking_us", "stream_ordered_us"):
        assert len(d[mode]) == 7 and all(v > 0 for v in d[mode].values())


# The reference's own programs (test/vector.c, examples/example.c) include
# only its public header.  Where the reference's sources are present (they
# are not on GPU machines) they must compile against include/vkhel/vkhel.h
# and link against libvkhel.so unchanged: the source-level drop-in check.
def _reference_src():
    from oracle import pyoracle
    return pyoracle.reference_dir()


REFERENCE_SRC = _reference_src()


@pytest.mark.skipif(REFERENCE_SRC is None or not os.path.isfile(os.path.join(REFERENCE_SRC, "test", "vector.c")),
                    reason="the reference's sources are not present on this machine")
@pytest.mark.parametrize("src", ["test/vector.c", "examples/example.c"])
def test_reference_programs_compile_and_link_unchanged(vk, tmp_path, src):
    from vkhel_gb300 import LIB_PATH
    libdir = os.path.dirname(LIB_PATH)
    exe = str(tmp_path / os.path.basename(src).replace(".c", ""))
    r = subprocess.run(["gcc", "-std=gnu11", "-O2", "-I", os.path.join(ROOT, "include", "vkhel"),
                        os.path.join(REFERENCE_SRC, src), "-o", exe, "-L", libdir, "-lvkhel",
                        f"-Wl,-rpath,{libdir}", "-Wl,--no-undefined"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "implicit declaration" not in r.stderr, r.stderr

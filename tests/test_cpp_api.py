"""The drop-in boundary from a C++ caller's side: a program written against the
reference's C++ solve API (tests/cpp/mehrotra_api.cpp, after the reference's
tests/unit/test_mehrotra.cu:13-79) compiles against include/ unchanged and links
the engine library; on a GPU it solves the reference's textbook LP. The CLI's
JSON keys come in the reference's order (tests/benchmark/sankhya_benchmark_cli.cpp:84-97)."""
import json
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
REFERENCE_KEYS = ["solver", "status", "execution_path", "fallback_triggered", "solve_time_ms", "iterations",
                  "objective", "primal_residual", "variables", "constraints", "nnz", "certificate_pass"]


def build_caller(sk, out_dir):
    exe = os.path.join(str(out_dir), "mehrotra_api")
    libdir = os.path.dirname(sk.LIB_PATH)
    cmd = ["g++", "-O1", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA, "include"),
           os.path.join(HERE, "cpp", "mehrotra_api.cpp"), "-o", exe, "-L" + libdir, "-lsankhya_gb300",
           "-Wl,-rpath," + libdir, "-L" + os.path.join(CUDA, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.join(CUDA, "lib64")]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    return exe


def test_reference_caller_compiles_and_links(sk, tmp_path):
    exe = build_caller(sk, tmp_path)
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
def test_reference_caller_solves_on_gpu(gpu, tmp_path):
    exe = build_caller(gpu, tmp_path)
    p = subprocess.run([exe], capture_output=True, text=True)
    assert p.returncode == 0, (p.stdout, p.stderr)
    res = json.loads(p.stdout.strip().splitlines()[-1])
    assert res["status"] == 0 and res["failures"] == 0 and abs(res["objective"] + 20.0) <= 1e-8


@pytest.mark.gpu
def test_cli_json_keys_in_reference_order(gpu):
    cli = os.path.join(os.path.dirname(gpu.LIB_PATH), "sankhya_cli")
    out = subprocess.run([cli, "--family", "0"], capture_output=True, text=True, check=True).stdout
    res = json.loads(out)
    keys = list(res.keys())
    assert keys[:len(REFERENCE_KEYS)] == REFERENCE_KEYS
    assert res["solver"] == "SANKHYA" and res["status"] == "Optimal" and res["certificate_pass"] is True

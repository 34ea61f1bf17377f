"""Host-side batch scheduling without a GPU: the step lists restricted to some LPs
of a batch (ipm::restrict_steps, used when a factorisation covers a few LPs of a
batch), checked by a C++ program against the full front plan of a dense-front and
a sparse multifrontal batch; and the sk_info / sk_options layouts of the ctypes
binding against the C header."""
import ctypes
import json
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def test_restricted_steps_match_the_plan(sk, tmp_path):
    exe = os.path.join(str(tmp_path), "front_plan_restrict")
    libdir = os.path.dirname(sk.LIB_PATH)
    cmd = ["g++", "-O1", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "soverign-gpu-accelerator-_gb300", "csrc"), "-I" + os.path.join(CUDA, "include"),
           os.path.join(HERE, "cpp", "front_plan_restrict.cpp"), "-o", exe, "-L" + libdir, "-lsankhya_gb300",
           "-Wl,-rpath," + libdir, "-L" + os.path.join(CUDA, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.join(CUDA, "lib64")]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    p = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, (p.stdout, p.stderr)
    res = json.loads(p.stdout.strip().splitlines()[-1])
    assert res["failed"] == 0 and res["checks"] > 1000
    # both plan kinds were exercised: one dense front per LP, and several levels of fronts
    assert res["dense"]["dense_mode"] == 1 and res["sparse"]["dense_mode"] == 0
    assert res["sparse"]["levels"] > 1


def _header_fields(struct):
    txt = open(os.path.join(ROOT, "include", "sankhya", "sk_ipm.h")).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (struct, struct), txt, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(?:const\s+)?(?:unsigned\s+)?(?:long\s+long|double|int|float|char)\s*\**\s*(.+)", decl)
        assert m, decl
        names += [n.strip().lstrip("*") for n in m.group(1).split(",")]
    return names


def test_info_and_options_bindings_follow_the_header(sk):
    assert [f for f, _ in sk.Info._fields_] == _header_fields("sk_info")
    assert [f for f, _ in sk.Options._fields_] == _header_fields("sk_options")
    # factorisation times per front precision are part of sk_info
    assert "factor_ms_fp32" in sk.Info.as_dict(sk.Info())
    # the default switch point of mixed precision
    opt = sk.Options()
    sk.lib().sk_options_default(ctypes.byref(opt))
    assert opt.mu_switch == 1e-4

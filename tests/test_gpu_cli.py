"""Drop-in at the C level: the reference's own command-line tool
(utils/zfp.c, unmodified) compiled against this repository's headers
(include/zfp.h, include/bitstream.h) and linked with libzfp_gb300.so,
run with `-x cuda`, must write the same compressed files and the same
decompressed arrays as the same tool built against the reference library
and run serially -- and must read the reference's files.  Header and ABI
compatibility of a C translation unit is what this shows; the tool reaches
the GPU only through zfp_stream_set_execution(zfp_exec_cuda).  Needs the
reference's sources (its checkout, or the copy staged from it) and gcc."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import pyoracle
from zfp_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WORK = os.path.join(ROOT, "tests", "native", "_build", "cli")


def build_tools():
    ref_src = pyoracle.reference_sources()
    if not ref_src or not shutil.which("gcc"):
        pytest.skip("the reference's sources or gcc are not available here")
    ref_lib = pyoracle.build_ref()
    if not ref_lib or not os.path.exists(ref_lib):
        pytest.skip("the reference library could not be built here")
    os.makedirs(WORK, exist_ok=True)
    cli = os.path.join(ref_src, "utils", "zfp.c")
    libdir = os.path.join(ROOT, "zfp_gb300")
    gpu = os.path.join(WORK, "zfp_gb300_cli")
    ref = os.path.join(WORK, "zfp_ref_cli")
    # the tool sees only this repository's headers (zfp.h and the zfp/...
    # paths it includes), as a program built against this library would
    cmds = [["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"),
             cli, "-o", gpu, "-L", libdir, "-lzfp_gb300", f"-Wl,-rpath,{libdir}", "-lm"],
            ["gcc", "-O2", "-std=c99", "-I", os.path.join(ref_src, "include"), cli, "-o", ref, ref_lib,
             f"-Wl,-rpath,{os.path.dirname(ref_lib)}", "-lm"]]
    for c in cmds:
        r = subprocess.run(c, capture_output=True, text=True)
        assert r.returncode == 0, f"{' '.join(c)}\n{r.stderr[-2000:]}"
    return gpu, ref


CASES = [  # dtype, shape (numpy order), mode arguments, header
    (np.float32, (40, 48, 56), ["-r", "8"], False),
    (np.float32, (40, 48, 56), ["-p", "20"], True),
    (np.float64, (33, 65, 70), ["-a", "1e-3"], True),
    (np.float32, (40, 48, 56), ["-R"], False),
    (np.float64, (300, 257), ["-r", "12"], True),
    (np.float32, (12, 10, 9, 11), ["-a", "1e-2"], True),
]


@pytest.mark.parametrize("dtype,shape,mode,header", CASES, ids=lambda v: str(v))
def test_reference_cli_on_gpu_matches_reference(lib, cuda, tmp_path, dtype, shape, mode, header):
    gpu, ref = build_tools()
    a = synth.smooth_field(shape, dtype, seed=4, noise=1e-2)
    inp = str(tmp_path / "in.raw")
    a.tofile(inp)
    typ = ["-f"] if dtype == np.float32 else ["-d"]
    dims = [f"-{len(shape)}"] + [str(v) for v in reversed(shape)]
    meta = typ + dims + mode + (["-h"] if header else [])
    out = {}
    for name, tool, extra in (("ref", ref, []), ("gpu", gpu, ["-x", "cuda"])):
        z, o = str(tmp_path / f"{name}.zfp"), str(tmp_path / f"{name}.out")
        r = subprocess.run([tool, "-q", "-i", inp, "-z", z, "-o", o] + meta + extra, capture_output=True, text=True)
        assert r.returncode == 0, f"{name}: {r.stderr}"
        out[name] = (open(z, "rb").read(), open(o, "rb").read())
    assert out["gpu"][0] == out["ref"][0], "compressed files differ"
    assert out["gpu"][1] == out["ref"][1], "decompressed arrays differ"
    # the GPU build reads the reference's compressed file (no block index: parsed on the GPU)
    o2 = str(tmp_path / "gpu2.out")
    args = ["-h"] if header else typ + dims + mode
    r = subprocess.run([gpu, "-q", "-x", "cuda", "-z", str(tmp_path / "ref.zfp"), "-o", o2] + args,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert open(o2, "rb").read() == out["ref"][1]

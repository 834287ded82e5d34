"""The oracle and the library's host code under AddressSanitizer and UndefinedBehaviorSanitizer.

tests/sanitize_driver.c exercises oracle/kmc_oracle.c (every entry point the tests use: tables,
neighbour lists, both hop paths, batched MSD, contacts mode, tracks, trim) and
cnt_film_monte_carlo_gb300/csrc/kmc_host.cpp (trim, domain, tables, the closed-form labeller,
the diffusion fit, the mesh reader), including their refusals (a link past the film, a grid
count that is NaN, fractional, negative or huge, a mesh file with a token that is not a number).  Compiled with -fsanitize=address,undefined and run with
halt_on_error: any out-of-bounds access, leak or undefined operation fails the test.  CPU only.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FLAGS = ["-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
         "-ffp-contract=off"]


def test_oracle_and_host_code_are_clean_under_sanitizers(tmp_path):
    if not (shutil.which("gcc") and shutil.which("g++")):
        pytest.skip("gcc/g++ not available")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "oracle"),
           "-I" + os.path.join(ROOT, "cnt_film_monte_carlo_gb300", "csrc")]
    objs = []
    for src, cc, std in ((os.path.join(ROOT, "oracle", "kmc_oracle.c"), "gcc", "-std=gnu11"),
                         (os.path.join(ROOT, "tests", "sanitize_driver.c"), "gcc", "-std=gnu11"),
                         (os.path.join(ROOT, "cnt_film_monte_carlo_gb300", "csrc", "kmc_host.cpp"), "g++", "-std=c++17")):
        o = str(tmp_path / (os.path.basename(src) + ".o"))
        r = subprocess.run([cc, std, *FLAGS, "-fopenmp", *inc, "-c", src, "-o", o], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        objs.append(o)
    exe = str(tmp_path / "sanitize_driver")
    r = subprocess.run(["g++", *FLAGS, "-fopenmp", "-o", exe, *objs, "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    mesh = tmp_path / "mesh"
    mesh.mkdir()
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:halt_on_error=1", UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1",
               OMP_NUM_THREADS="1")
    r = subprocess.run([exe, str(mesh)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert "sanitize_driver: ok" in r.stdout
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr

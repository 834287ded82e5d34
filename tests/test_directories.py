"""The drop-in driver's output and input directory helpers, in both mirrors.

The reference prepares its output directory with prepare_directory and checks the mesh input
directory with check_directory (src/helper/prepare_directory.hpp:8-105, called from
monte_carlo.h:131,135).  What they do:
  * a missing output directory is created;
  * a non-empty output directory is renamed to <dir>.N, the first N not taken, and a new empty
    one is made in its place;
  * with "keep old results" false the old one is deleted instead;
  * a path that exists but is not a directory is refused;
  * the checked input directory must exist, be a directory, and be non-empty unless it should
    be empty;
  * a leading '~' is replaced by $HOME.
The Python class (monte_carlo.py) and the C++ class (csrc/monte_carlo.hpp, through a small
helper compiled with g++) must both behave this way.
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

from cnt_film_monte_carlo_gb300 import monte_carlo as M

REPO = Path(__file__).resolve().parents[1]

NOT_ACCEPTABLE = "The input value for output directory is not acceptable."
NOT_EXISTS = "directory does NOT exists!!!"
NOT_DIR = "input path is NOT a directory!!!"
EMPTY = "directory is empty!!!"


@pytest.fixture(scope="module")
def cpp_exe(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("dirs") / "dirs_from_cpp"
    subprocess.run(
        ["g++", "-std=c++17", "-O1", "-I", str(REPO / "cnt_film_monte_carlo_gb300" / "csrc"),
         "-I", str(REPO / "include"), str(REPO / "tests" / "dirs_from_cpp.cpp"), "-o", str(exe)],
        check=True)
    return exe


class PyMirror:
    def prepare(self, path, keep=True):
        return M.prepare_directory(str(path), keep)

    def check(self, path, should_be_empty=False):
        return M.check_directory(str(path), should_be_empty)


class CppMirror:
    def __init__(self, exe):
        self.exe = exe

    def _run(self, op, path, flag):
        p = subprocess.run([str(self.exe), op, str(path), "1" if flag else "0"], capture_output=True, text=True,
                           env=os.environ.copy())
        out = p.stdout.strip()
        if p.returncode == 1 and out.startswith("error: "):
            raise ValueError(out[len("error: "):])
        assert p.returncode == 0, (p.returncode, p.stdout, p.stderr)
        return out

    def prepare(self, path, keep=True):
        return self._run("prepare", path, keep)

    def check(self, path, should_be_empty=False):
        return self._run("check", path, should_be_empty)


@pytest.fixture(params=["python", "cpp"])
def mirror(request):
    if request.param == "python":
        return PyMirror()
    return CppMirror(request.getfixturevalue("cpp_exe"))


def test_missing_output_directory_is_created(mirror, tmp_path):
    out = tmp_path / "a" / "b"
    assert mirror.prepare(out) == str(out)
    assert out.is_dir() and not any(out.iterdir())


def test_empty_output_directory_is_kept_in_place(mirror, tmp_path):
    out = tmp_path / "out"
    out.mkdir()
    mirror.prepare(out)
    assert out.is_dir() and not (tmp_path / "out.1").exists()


def test_old_results_are_renamed_to_the_first_free_number(mirror, tmp_path):
    out = tmp_path / "out"
    out.mkdir()
    (out / "run1.dat").write_text("1")
    (tmp_path / "out.1").mkdir()  # taken: the next free number is 2
    mirror.prepare(out, True)
    assert out.is_dir() and not any(out.iterdir())
    assert (tmp_path / "out.2" / "run1.dat").read_text() == "1"
    (out / "run2.dat").write_text("2")
    mirror.prepare(out, True)
    assert (tmp_path / "out.3" / "run2.dat").read_text() == "2"
    assert not any(out.iterdir())


def test_old_results_are_deleted_when_not_kept(mirror, tmp_path):
    out = tmp_path / "out"
    (out / "sub").mkdir(parents=True)
    (out / "sub" / "x.dat").write_text("x")
    mirror.prepare(out, False)
    assert out.is_dir() and not any(out.iterdir())
    assert sorted(p.name for p in tmp_path.iterdir()) == ["out"]


def test_output_path_that_is_a_file_is_refused(mirror, tmp_path):
    f = tmp_path / "file"
    f.write_text("not a directory")
    with pytest.raises(ValueError, match=NOT_ACCEPTABLE.replace(".", r"\.")):
        mirror.prepare(f)
    assert f.read_text() == "not a directory"


def test_checked_input_directory(mirror, tmp_path):
    with pytest.raises(ValueError, match=NOT_EXISTS.replace("!", r"\!")):
        mirror.check(tmp_path / "missing")
    f = tmp_path / "file"
    f.write_text("x")
    with pytest.raises(ValueError, match=NOT_DIR.replace("!", r"\!")):
        mirror.check(f)
    empty = tmp_path / "empty"
    empty.mkdir()
    with pytest.raises(ValueError, match=EMPTY.replace("!", r"\!")):
        mirror.check(empty)
    assert mirror.check(empty, True) == str(empty)
    full = tmp_path / "mesh"
    full.mkdir()
    (full / "tube_0.dat").write_text("0")
    assert mirror.check(full) == str(full)
    assert mirror.check(full, True) == str(full)  # the reference does not refuse a full one here


def test_leading_tilde_is_home(mirror, tmp_path, monkeypatch):
    home = tmp_path / "home"
    home.mkdir()
    monkeypatch.setenv("HOME", str(home))
    assert mirror.prepare("~/out") == f"{home}/out"
    assert (home / "out").is_dir()
    # "~x" is $HOME followed by "x", not the home of a user named x
    assert mirror.prepare("~x") == f"{home}x"
    assert Path(f"{home}x").is_dir()
    (home / "out" / "f").write_text("f")
    assert mirror.check("~/out") == f"{home}/out"


@pytest.mark.parametrize("literal", ["NaN", "Infinity", "-Infinity"])
def test_python_driver_refuses_non_json_numbers(tmp_path, literal):
    # input.json is refused before anything else happens (no device needed), as cntkmc_run's
    # reader refuses it
    p = tmp_path / "input.json"
    p.write_text('{"exciton monte carlo": {"monte carlo time step": %s}}' % literal)
    with pytest.raises(ValueError, match="not a JSON number"):
        M.run(str(p))


@pytest.mark.parametrize("dt", [0.0, -1e-15, float("nan"), float("inf"), 1e-40])
def test_time_steps_that_never_reach_the_end_are_refused(dt):
    # main.cpp's `while (time < max time) { time += dt; ... }` never ends for these steps; the
    # driver refuses them instead of looping (a NaN step would compare false and run 0 steps in
    # the reference's loop, but it is refused here too)
    sim = object.__new__(M.monte_carlo)
    sim._time = 0.0
    with pytest.raises(ValueError, match="time step"):
        sim.steps_until(1e-12, dt)


def test_time_step_stuck_on_a_large_clock_is_refused():
    sim = object.__new__(M.monte_carlo)
    sim._time = 1.0  # 1e-20 s is below half an ulp of 1 s: the sum stays at 1.0
    with pytest.raises(ValueError, match="time step"):
        sim.steps_until(1.0 + 1e-9, 1e-20)


def test_step_count_follows_the_reference_accumulation():
    sim = object.__new__(M.monte_carlo)
    sim._time = 0.0
    n, t = 0, 0.0
    while t < 1e-12:
        t += 1e-15
        n += 1
    assert sim.steps_until(1e-12, 1e-15) == n
    assert sim.steps_until(0.0, 1e-15) == 0

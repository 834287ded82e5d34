"""The drop-in driver's JSON reader/writer (csrc/json_lite.hpp) against Python's json.

The driver reads the reference's input.json (main.cpp:32-54 reads it with nlohmann::json) and
writes the properties back beside its outputs (save_json_properties, monte_carlo.h:319-324).  A small
helper compiled with g++ parses a file and writes it back; Python's json must read the same
value out of the result, and malformed files must be refused.
"""
import json
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]

GOOD = [
    {"mode": "contacts", "number of segments": 5, "temperature [kelvin]": 300.0},
    {"a": [1, -2, 3.5, 1e-9, 6.02214076e23, -0.0], "b": {"c": {"d": []}, "e": {}}},
    {"flags": [True, False, None], "empty": "", "nested": [[[]], [{}]]},
    {'quote " and backslash \\': 'path\\to\\"file"', "tab\tnew\nline": "\r\b\f\x01\x1f"},
    {"unicode": "é中\U0001f600", "slash": "a/b"},
    [0.1, 0.2, 0.30000000000000004, 2.2250738585072014e-308, 1.7976931348623157e308],
    "just a string",
    42,
]

BAD = [
    "",
    "{",
    '{"a": }',
    '{"a" 1}',
    "[1, 2",
    '"unterminated',
    '{"a": 1} x',
    '"\\u12"',
    '"\\ud83d\\u0041"',
    "nul",
    # numbers outside the JSON grammar
    "nan", "NaN", "inf", "-Infinity", "-", "01", "-01", "+1", ".5", "1.", "1e", "1e+", "0x10", "1.5.2",
    # escapes and characters JSON strings do not allow
    '"\\q"', '"\\x41"', '"\\ud83d"', '"\\ud83d x"', '"\\udc00"', '"a\x01b"', '"tab\there"',
]


@pytest.fixture(scope="module")
def roundtrip(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("jl") / "json_roundtrip"
    subprocess.run(
        ["g++", "-std=c++17", "-O1", "-I", str(REPO / "cnt_film_monte_carlo_gb300" / "csrc"),
         str(REPO / "tests" / "json_roundtrip.cpp"), "-o", str(exe)],
        check=True)
    return exe


def run(exe, tmp_path, text):
    p = tmp_path / "in.json"
    p.write_bytes(text.encode("utf-8"))
    return subprocess.run([str(exe), str(p)], capture_output=True)


@pytest.mark.parametrize("value", GOOD, ids=range(len(GOOD)))
def test_round_trip(roundtrip, tmp_path, value):
    for text in (json.dumps(value), json.dumps(value, indent=2, ensure_ascii=False)):
        r = run(roundtrip, tmp_path, text)
        assert r.returncode == 0, r.stderr
        back = json.loads(r.stdout.decode("utf-8"))
        assert back == value
        # a second pass is a fixed point of the writer
        r2 = run(roundtrip, tmp_path, r.stdout.decode("utf-8"))
        assert r2.returncode == 0 and r2.stdout == r.stdout


def test_numbers_exact(roundtrip, tmp_path):
    vals = [1.0 / 3.0, 1e-300, 123456789.123456789, 5e-324, -2.5e-12]
    r = run(roundtrip, tmp_path, json.dumps(vals))
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout) == vals


def test_numbers_keep_their_text(roundtrip, tmp_path):
    """A number is written back as it was read: integers stay integers, floats stay floats (0.0,
    2.0, 1e-15 and -0.0 are not turned into 0, 2 or 1.0000000000000001e-15), and integers past
    2^53 keep every digit."""
    text = "[0, 0.0, -0.0, 2.0, 1e-15, 1E+3, 0.1, 12345678901234567890, -7]"
    r = run(roundtrip, tmp_path, text)
    assert r.returncode == 0, r.stderr
    assert r.stdout.decode().strip() == text
    back = json.loads(r.stdout)
    assert [type(x) for x in back] == [int, float, float, float, float, float, float, int, int]
    assert back[7] == 12345678901234567890


@pytest.mark.parametrize("text", BAD, ids=range(len(BAD)))
def test_malformed_refused(roundtrip, tmp_path, text):
    r = run(roundtrip, tmp_path, text)
    assert r.returncode == 2, (text, r.stdout, r.stderr)
    assert b"json:" in r.stderr


def test_random_documents_round_trip(roundtrip, tmp_path_factory):
    """Random JSON documents (nested objects and arrays, unicode strings with escapes, finite
    doubles including subnormals and -0.0, integers up to 2^53) read back equal after one pass
    through the C++ reader and writer."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    d = tmp_path_factory.mktemp("jl_random")
    text_st = st.text(st.characters(exclude_categories=("Cs",)), max_size=12)
    scalars = (st.none() | st.booleans() | st.integers(-(2**53), 2**53)
               | st.floats(allow_nan=False, allow_infinity=False) | text_st)
    docs = st.recursive(scalars, lambda c: st.lists(c, max_size=5) | st.dictionaries(text_st, c, max_size=5),
                        max_leaves=25)

    @hyp.settings(max_examples=150, deadline=None, database=None, derandomize=True)
    @hyp.given(docs)
    def check(value):
        text = json.dumps(value, ensure_ascii=False)
        r = run(roundtrip, d, text)
        assert r.returncode == 0, (text, r.stderr)
        back = json.loads(r.stdout.decode("utf-8"))
        assert back == value
        assert json.dumps(back, sort_keys=True) == json.dumps(value, sort_keys=True)  # -0.0 and key sets

    check()


@pytest.mark.parametrize("raw", [b"\x80", b"\xc0\xaf", b"\xc3", b"\xe0\x80\xaf", b"\xed\xa0\x80",
                                 b"\xf4\x90\x80\x80", b"\xf5\x80\x80\x80", b"\xff", b"\xe2\x82"])
def test_invalid_utf8_in_strings_is_refused(roundtrip, tmp_path, raw):
    # stray continuation, overlong, truncated, surrogate (U+D800), above U+10FFFF, never-valid bytes
    p = tmp_path / "in.json"
    p.write_bytes(b'{"a": "x' + raw + b'y"}')
    r = subprocess.run([str(roundtrip), str(p)], capture_output=True)
    assert r.returncode == 2 and b"UTF-8" in r.stderr, (raw, r.returncode, r.stderr)


def test_valid_utf8_edges_are_read(roundtrip, tmp_path):
    s = "\u0080\u07ff\u0800\ud7ff\ue000\uffff\U00010000\U0010ffff"
    p = tmp_path / "in.json"
    p.write_bytes(json.dumps({"a": s}, ensure_ascii=False).encode("utf-8"))
    r = subprocess.run([str(roundtrip), str(p)], capture_output=True)
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout.decode("utf-8")) == {"a": s}


def test_nesting_depth_is_bounded(roundtrip, tmp_path):
    """512 levels of objects or arrays are read; deeper files are refused with a message instead
    of overflowing the stack of the recursive reader."""
    r = run(roundtrip, tmp_path, "[" * 512 + "]" * 512)
    assert r.returncode == 0 and json.loads(r.stdout) is not None
    r = run(roundtrip, tmp_path, '{"a":' * 512 + "1" + "}" * 512)
    assert r.returncode == 0
    for text in ("[" * 513 + "]" * 513, "[" * 200000 + "]" * 200000, '{"a":' * 100000):
        r = run(roundtrip, tmp_path, text)
        assert r.returncode == 2 and b"nested too deep" in r.stderr, (len(text), r.returncode)


def test_arbitrary_bytes_are_read_or_refused(roundtrip, tmp_path_factory):
    """Any file is either a JSON document (exit 0, and Python's json reads the same value out of
    the writer's output) or refused with a message (exit 2): never a crash."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    d = tmp_path_factory.mktemp("jl_bytes")
    pieces = st.sampled_from(['{', '}', '[', ']', ',', ':', '"', '\\', 'u', 'd83d', 'e', '-', '+', '.', '0', '1',
                              '9', 'true', 'false', 'null', ' ', '\n', 'NaN', '\x00', '\x1f', 'é', '\udc00'])
    texts = st.lists(pieces, max_size=40).map("".join) | st.binary(max_size=60).map(
        lambda b: b.decode("latin-1"))

    @hyp.settings(max_examples=300, deadline=None, database=None, derandomize=True)
    @hyp.given(texts)
    def check(text):
        p = d / "in.json"
        p.write_bytes(text.encode("utf-8", "surrogatepass"))
        r = subprocess.run([str(roundtrip), str(p)], capture_output=True)
        assert r.returncode in (0, 2), (text, r.returncode, r.stderr)
        if r.returncode == 0:
            back = json.loads(r.stdout.decode("utf-8"))
            assert back == json.loads(text.encode("utf-8", "surrogatepass").decode("utf-8"))

    check()


@pytest.mark.parametrize("text,mode,expect", [
    ("3.9", "int", b"3"), ("-3.9", "int", b"-3"), ("1e18", "int", b"1000000000000000000"),
    ("1e999", "int", None), ("-1e999", "int", None), ("9.3e18", "int", None), ('"7"', "int", None),
    ("2147483647", "int32", b"2147483647"), ("-2147483648", "int32", b"-2147483648"),
    ("2147483648", "int32", None), ("-2147483649", "int32", None), ("1e10", "int32", None),
])
def test_integer_conversions_are_range_checked(roundtrip, tmp_path, text, mode, expect):
    # the driver reads counts (particles, sections, segments, tracked particles) through these:
    # a value outside the integer's range is refused, not converted with undefined behaviour
    p = tmp_path / "in.json"
    p.write_text(text)
    r = subprocess.run([str(roundtrip), str(p), mode], capture_output=True)
    if expect is None:
        assert r.returncode == 2 and b"json:" in r.stderr, (text, mode, r.returncode, r.stdout)
    else:
        assert r.returncode == 0 and r.stdout.strip() == expect, (text, mode, r.stdout, r.stderr)

"""Regenerate the exciton-physics fixtures tests/golden/ref_et_*.npz from the reference's own code.

The reference ships no tests or golden values for its exciton physics, so the fixtures are the
outputs of src/exciton_transfer/cnt.cpp and exciton_transfer.cpp themselves, compiled unchanged
against the project's second Armadillo shim (oracle/shim_et/armadillo) into
oracle/_ref/ref_exciton by ``make -C oracle ref``.  For each donor/acceptor pair of tubes the
fixture holds, per tube, the lattice and K2-extended parameters, unit-cell positions, bands,
valleys, relevant-state windows, vq, PI, eps and the three A-exciton dispersions; for the pair,
the thermally relevant A2-singlet states, the matched state pairs of the first geometry with
|Q|, J and M, and the first-order transfer rate at every geometry.

Needs the reference sources: set CNT_REFERENCE_DIR to the reference checkout (the script stops
with a message when it is unset).  Run: CNT_REFERENCE_DIR=<checkout> python
tests/golden/make_golden_exciton.py [case ...]
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

NM = 1e-9
# (donor n, m, cells), (acceptor n, m, cells), geometries (z_shift m, axis shift 1 m, axis shift 2 m,
# theta rad).  42/42 and 42/65 are the pairs of the reference's own input.json ("exciton
# transfer" sections, z_shift 1.9 nm, angles 0-90 deg); 75/84 mixes two of the surrogate's
# chiralities.
CASES = {
    "ref_et_42_42": ((4, 2, 10), (4, 2, 10), [(1.9 * NM, 0, 0, 0.0), (1.9 * NM, 0, 0, 0.5), (1.9 * NM, 0, 0, 1.2),
                                              (1.9 * NM, 0, 0, np.pi / 2), (3 * NM, 1 * NM, -1 * NM, 0.3),
                                              (6 * NM, 2 * NM, 0, 2.5)]),
    "ref_et_42_65": ((4, 2, 10), (6, 5, 3), [(1.9 * NM, 0, 0, 0.0), (1.9 * NM, 0, 0, 0.7), (4 * NM, 0.5 * NM, 0, 1.0)]),
    "ref_et_84_84": ((8, 4, 12), (8, 4, 12), [(1.5 * NM, 0, 0, 0.0), (3 * NM, 0, 0, 0.0), (6 * NM, 0, 0, 0.0),
                                              (2 * NM, 1 * NM, 1 * NM, 0.8)]),
    "ref_et_75_84": ((7, 5, 3), (8, 4, 12), [(1.5 * NM, 0, 0, 0.0), (2.5 * NM, 0, 0, 0.4)]),
}


def read_dump(path: str) -> dict:
    """Records of oracle/ref_exciton.cpp: u32 name length, name, u8 kind (0 f64, 1 c128, 2 i64),
    u32 ndim, u64 dims, data (row-major)."""
    out = {}
    with open(path, "rb") as f:
        b = f.read()
    i = 0
    while i < len(b):
        (nl,) = struct.unpack_from("<I", b, i)
        i += 4
        name = b[i:i + nl].decode()
        i += nl
        kind = b[i]
        i += 1
        (nd,) = struct.unpack_from("<I", b, i)
        i += 4
        dims = struct.unpack_from("<%dQ" % nd, b, i)
        i += 8 * nd
        dt = {0: np.float64, 1: np.complex128, 2: np.int64}[kind]
        n = int(np.prod(dims)) if nd else 1
        sz = n * np.dtype(dt).itemsize
        out[name] = np.frombuffer(b[i:i + sz], dtype=dt).reshape(dims).copy()
        i += sz
    return out


def make_case(name, donor, acceptor, geos, tmp):
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_exciton")
    path = os.path.join(tmp, name + ".bin")
    args = [exe, path, *(str(x) for x in donor + acceptor)]
    for g in geos:
        args += [repr(float(x)) for x in g]
    r = subprocess.run(args, capture_output=True, text=True, env=dict(os.environ, KMC_REF_SCRATCH=tmp), timeout=1200)
    if r.returncode != 0:
        raise RuntimeError(f"ref_exciton failed:\n{r.stdout}\n{r.stderr}")
    d = read_dump(path)
    if donor == acceptor:  # one tube: its records appear once
        d = {k: v for k, v in d.items() if not k.startswith("a_")}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(name, r.stdout.strip())


def main(names=()):
    ref_dir = O.reference_dir()
    if ref_dir is None:
        sys.exit("make_golden_exciton.py: set CNT_REFERENCE_DIR to the reference checkout")
    O.build(ref_dir)
    with tempfile.TemporaryDirectory() as tmp:
        for name, (d, a, g) in CASES.items():
            if not names or name in names:
                make_case(name, d, a, g, tmp)


if __name__ == "__main__":
    main(sys.argv[1:])

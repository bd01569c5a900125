"""The drop-in classes' on-disk format, on the CPU: a matrix filled by the
drop-in generators and written with Matrix*::write is, byte for byte, the
oracle's restatement of the reference's writer (MatrixCSR.cpp:179-204 and its
siblings) applied to the oracle's own fill of the same matrix; reading the
file back (Matrix*::read, MatrixCSR.cpp:206-232) and writing again gives the
same bytes.  Every format, the three generators, one-block and 2-D block
positions."""
import os
import subprocess

import pytest

from oracle.oracle import parse_binary, write_binary

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
FORMATS = ["COO", "SCOO", "CSR", "ELL", "DENSE"]
CASES = [("cqmat", 40, 40, 6, 0.1, 3, (0, 0, 1, 1)), ("cqmat", 30, 50, 9, 0.5, 1, (1, 0, 2, 3)),
         ("cdiag", 40, 40, 3, 0.0, 0, (0, 0, 1, 1)), ("cdiag", 25, 31, 2, 0.0, 0, (1, 1, 2, 2)),
         ("stochastic", 36, 36, 5, 0.2, 2, (0, 1, 2, 2)), ("cqmat", 1000, 1000, 12, 0.1, 0, (0, 0, 1, 1))]


@pytest.fixture(scope="module")
def prog(capi, tmp_path_factory):
    lib_dir = os.path.dirname(capi.LIB_PATH)
    out = str(tmp_path_factory.mktemp("dropin") / "dropin_files")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", f"-I{INCLUDE}",
           os.path.join(ROOT, "tests", "cpp", "dropin_files.cpp"), f"-L{lib_dir}", "-ltbsla_gb300",
           f"-Wl,-rpath,{lib_dir}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return out


@pytest.mark.parametrize("fmt", FORMATS)
def test_written_files_match_the_reference_layout(prog, orc, tmp_path, fmt):
    for (gen, nr, nc, c, q, seed, blk) in CASES:
        if fmt == "DENSE" and nr > 100:
            continue
        first, second = tmp_path / "first.bin", tmp_path / "second.bin"
        r = subprocess.run([prog, fmt, gen, str(nr), str(nc), str(c), repr(q), str(seed), *map(str, blk),
                            str(first), str(second)], capture_output=True, text=True)
        assert r.returncode == 0, (fmt, gen, r.stderr)
        if gen == "cqmat":
            o = orc.fill_cqmat(fmt, nr, nc, c, q, seed, *blk)
        elif gen == "cdiag":
            o = orc.fill_cdiag(fmt, nr, nc, c, *blk)
        else:
            o = orc.fill_cqmat_stochastic(fmt, nr, nc, c, q, seed, *blk)
        want = write_binary(o.arrays)
        got = first.read_bytes()
        assert got == want, (fmt, gen, nr, nc, c, q, seed, blk, len(got), len(want))
        assert second.read_bytes() == got, (fmt, gen, "read back")


MM_FILES = {
    "general": "%%MatrixMarket matrix coordinate real general\n% a comment\n% another\n5 4 7\n"
               "1 1 1.5\n2 3 -2.25\n5 4 3e-3\n3 2 7\n1 4 -1\n4 1 0.5\n2 3 1\n",
    "symmetric": "%%MatrixMarket matrix coordinate real symmetric\n6 6 6\n1 1 4\n2 1 -1\n3 2 -1\n"
                 "4 4 2.5\n6 3 8\n6 6 1e-7\n",
    "short": "%%MatrixMarket matrix coordinate real general\n3 3 5\n1 1 1\n2 2 2\n",
    "pattern": "%%MatrixMarket matrix coordinate pattern general\n3 3 2\n1 1\n2 2\n",
    "array": "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",
    "skew": "%%MatrixMarket matrix coordinate real skew-symmetric\n3 3 1\n2 1 1\n",
}


@pytest.mark.parametrize("kind", sorted(MM_FILES))
def test_matrix_market_matches_reference(prog, ref, tmp_path, kind):
    """MatrixCOO::readMM of the drop-in class gives the reference's matrix
    byte for byte (its binary file), general and symmetric files, a file
    with fewer entries than it declares; both refuse the other kinds."""
    path = tmp_path / f"{kind}.mtx"
    path.write_text(MM_FILES[kind])
    out = tmp_path / "mm.bin"
    r = subprocess.run([prog, "MM", str(path), str(out)], capture_output=True, text=True)
    rm = ref.read_mm(str(path))
    if rm is None:
        assert r.returncode == 6, (kind, r.returncode, r.stderr)
        return
    assert r.returncode == 0, (kind, r.stderr)
    assert out.read_bytes() == rm.serialized(), kind


@pytest.mark.parametrize("fmt", ["CSR", "ELL", "SCOO", "DENSE"])
def test_conversions_match_reference(prog, ref, tmp_path, fmt):
    """The drop-in classes' constructors from a MatrixCOO (MatrixCSR.cpp:29-74,
    MatrixELL.cpp:12-54, MatrixSCOO.cpp:53-68, MatrixDENSE.cpp:11-28) and
    MatrixCOO::normalize_columns give the reference's matrices byte for byte
    (repeated entries, q = 1 fills, empty and rectangular shapes)."""
    for (nr, nc, c, q, seed) in [(40, 40, 6, 0.1, 3), (30, 50, 9, 0.5, 1), (50, 20, 4, 1.0, 2), (12, 12, 0, 0.0, 0),
                                 (200, 200, 11, 0.3, 5)]:
        for norm in (0, 1):
            out = tmp_path / "conv.bin"
            r = subprocess.run([prog, "CONV", fmt, str(nr), str(nc), str(c), repr(q), str(seed), str(norm), str(out)],
                               capture_output=True, text=True)
            assert r.returncode == 0, (fmt, r.stderr)
            coo = ref.fill_cqmat("COO", nr, nc, c, q, seed)
            empty = parse_binary("COO", coo.serialized()).values.size == 0
            if norm:
                coo.normalize_columns()
            want = coo.convert(fmt).serialized()
            got = out.read_bytes()
            if empty:
                # a fill that stores nothing leaves the reference's nnz unset (the converted
                # matrices copy it): every other byte agrees
                got, want = got[:24] + got[32:], want[:24] + want[32:]
            assert got == want, (fmt, nr, nc, c, q, seed, norm, len(got), len(want))

"""The reference's text formats: files written by libvissgb.so are byte-identical
to what the reference's `file << value << std::endl` writes
(vissGen10M_shade.cu:575-577, shade1M.cu:118-121, MIncline:425), and the reader
follows its `while (file >> a >> b ...)` loops."""
import ctypes as C
import subprocess

import numpy as np
import pytest

OSTREAM_SRC = r"""
#include <cstdio>
#include <fstream>
#include <vector>
int main(int argc, char** argv) {
  // argv: in.bin ncols out.txt ; floats row-major
  FILE* f = std::fopen(argv[1], "rb");
  std::vector<float> v;
  float x;
  while (std::fread(&x, 4, 1, f) == 1) v.push_back(x);
  std::fclose(f);
  int nc = std::atoi(argv[2]);
  std::ofstream o(argv[3]);
  for (size_t i = 0; i < v.size(); i += nc) {
    for (int c = 0; c < nc; ++c) { o << v[i + c]; if (c + 1 < nc) o << " "; }
    o << std::endl;
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def ostream_writer(tmp_path_factory):
    d = tmp_path_factory.mktemp("ostream")
    src = d / "w.cpp"
    src.write_text(OSTREAM_SRC.replace("#include <vector>", "#include <vector>\n#include <cstdlib>"))
    exe = d / "w"
    subprocess.run(["g++", "-O1", "-o", str(exe), str(src)], check=True)
    return exe


@pytest.fixture(scope="module")
def L():
    from viss_recon_shade_gb300 import _lib
    return _lib


def sample_values(n=5000, seed=0):
    rng = np.random.default_rng(seed)
    v = np.concatenate([rng.normal(0, 1, n), rng.normal(0, 1e4, n), np.ceil(rng.normal(0, 3000, n)),
                        rng.lognormal(0, 3, n), [0.0, -0.0, 1e-30, -1e30, 123456.0, 1234567.0, 0.1, 240.0]])
    return v.astype(np.float32)


@pytest.mark.parametrize("ncols", [1, 3, 4])
def test_float_files_byte_identical_to_ostream(L, ostream_writer, tmp_path, ncols):
    v = sample_values()
    v = v[: (v.size // ncols) * ncols]
    rows = v.reshape(-1, ncols)
    (tmp_path / "in.bin").write_bytes(rows.astype(np.float32).tobytes())
    ref = tmp_path / "ref.txt"
    subprocess.run([str(ostream_writer), str(tmp_path / "in.bin"), str(ncols), str(ref)], check=True)
    cols = np.ascontiguousarray(rows.T)
    out = tmp_path / "ours.txt"
    assert L.lib.viss_text_write_floats(str(out).encode(), ncols, C.c_void_p(cols.ctypes.data), rows.shape[0],
                                       rows.shape[0]) == 0
    assert out.read_bytes() == ref.read_bytes()


def test_int_files_as_the_shade_writer(L, ostream_writer, tmp_path):
    rng = np.random.default_rng(1)
    raw = rng.integers(1, 62821, (3000, 4)).astype(np.int32)
    (tmp_path / "in.bin").write_bytes(raw.astype(np.float32).tobytes())
    ref = tmp_path / "ref.txt"
    subprocess.run([str(ostream_writer), str(tmp_path / "in.bin"), "4", str(ref)], check=True)
    out = tmp_path / "ours.txt"
    assert L.lib.viss_text_write_ints(str(out).encode(), 4, C.c_void_p(raw.ctypes.data), raw.shape[0]) == 0
    assert out.read_bytes() == ref.read_bytes()
    back = np.zeros_like(raw)
    n = C.c_int64()
    assert L.lib.viss_text_read_ints(str(out).encode(), 4, C.c_void_p(back.ctypes.data), raw.shape[0], C.byref(n)) == 0
    assert n.value == raw.shape[0] and np.array_equal(back, raw)


def test_reader_header_and_columns(L, tmp_path):
    p = tmp_path / "l.txt"
    p.write_text("4\n0.5\n-0.25\n1e-3\n+2\n")
    out = np.zeros(8, np.float32)
    n, hv = C.c_int64(), C.c_int64()
    assert L.lib.viss_text_read_floats(str(p).encode(), 1, 1, C.c_void_p(out.ctypes.data), 8, C.byref(n),
                                       C.byref(hv)) == 0
    assert hv.value == 4 and n.value == 4
    assert out[:4].tolist() == [0.5, -0.25, np.float32(1e-3), 2.0]
    # 4-column uvw file with a truncated last row: the reference's loop stops there
    q = tmp_path / "updated_uvw1frequency10M.txt"
    q.write_text("1 2 3 4\n-5 6 -7 8\n9 10\n")
    cols = np.zeros(4 * 3, np.float32)
    assert L.lib.viss_text_read_floats(str(q).encode(), 0, 4, C.c_void_p(cols.ctypes.data), 3, C.byref(n),
                                       None) == 0
    assert n.value == 2
    assert cols.reshape(4, 3)[:, :2].T.tolist() == [[1, 2, 3, 4], [-5, 6, -7, 8]]


def test_large_file_parallel_parse_roundtrip(L, tmp_path):
    v = sample_values(200000, seed=3)
    out = tmp_path / "big.txt"
    assert L.lib.viss_text_write_floats(str(out).encode(), 1, C.c_void_p(v.ctypes.data), v.size, v.size) == 0
    back = np.zeros_like(v)
    n = C.c_int64()
    assert L.lib.viss_text_read_floats(str(out).encode(), 0, 1, C.c_void_p(back.ctypes.data), v.size, C.byref(n),
                                       None) == 0
    assert n.value == v.size
    # "%g" keeps 6 significant digits
    assert np.allclose(back, v, rtol=6e-6, atol=0)


def test_missing_file_is_an_io_error(L, tmp_path):
    n = C.c_int64()
    assert L.lib.viss_text_read_floats(str(tmp_path / "nope.txt").encode(), 0, 1, None, 0, C.byref(n), None) == \
        L.VISS_ERR_IO

"""The HDF5 subset (include/ppf_h5.h): round trips, a file written by real
libhdf5, and the failure modes the reference ignores."""
import glob
import os

import numpy as np
import pytest

import phasefield_coarsening_gb300 as ppf


def _fields(shape, seed=0):
    rng = np.random.default_rng(seed)
    return {n: rng.random(shape) for n in ("etaS", "etaL", "c")}


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("chunk", [None, (2, 3, 4), (1, 1, 1), (5, 6, 7)])
def test_round_trip(tmp_path, dtype, chunk):
    shape = (5, 6, 7)
    f = _fields(shape)
    p = str(tmp_path / "a.h5")
    ppf.h5_write(p, f, dtype=dtype, chunk=chunk)
    for n, a in f.items():
        got = ppf.h5_read(p, "/" + n)
        ref = a if dtype == "f64" else a.astype(np.float32).astype(np.float64)
        assert np.array_equal(got, ref)
        assert ppf.h5_dims(p, n) == shape


def test_chunked_multilevel_btree(tmp_path):
    # 9*8*9 = 648 chunks > 64 per node: a two-level chunk B-tree
    shape = (9, 8, 9)
    f = _fields(shape, 3)
    p = str(tmp_path / "m.h5")
    ppf.h5_write(p, f, chunk=(1, 1, 1))
    for n, a in f.items():
        assert np.array_equal(ppf.h5_read(p, n), a)


def test_mpi_layout_chunk_equals_subdomain(tmp_path):
    # the reference's MPI writer: chunk = subdomain NN/NQ (phasefield.c:577-579)
    shape = (12, 12, 12)
    f = _fields(shape, 5)
    p = str(tmp_path / "mpi.h5")
    ppf.h5_write(p, f, chunk=(6, 6, 6))
    for n, a in f.items():
        assert np.array_equal(ppf.h5_read(p, n), a)


def test_file_layout_is_hdf5_superblock_v0(tmp_path):
    p = str(tmp_path / "s.h5")
    ppf.h5_write(p, _fields((2, 2, 2)))
    b = open(p, "rb").read()
    assert b[:8] == b"\x89HDF\r\n\x1a\n" and b[8] == 0
    assert int.from_bytes(b[40:48], "little") == len(b)      # end-of-file address
    for sig in (b"HEAP", b"TREE", b"SNOD"):
        assert sig in b


def _libhdf5_file():
    try:
        import scipy
    except ImportError:
        return None
    c = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data",
                               "testhdf5_7.4_GLNX86.mat"))
    return c[0] if c else None


def test_reads_structure_of_file_written_by_libhdf5():
    """A MATLAB v7.3 file (libhdf5, 512-byte user block): the symbol-table
    walk must find its dataset and report its rank-2 shape as unsupported."""
    p = _libhdf5_file()
    if p is None:
        pytest.skip("scipy test data not installed")
    with pytest.raises(ppf.PPFError) as e:
        ppf.h5_dims(p, "testdouble")
    assert e.value.code == -4 and "rank 2" in str(e.value)
    with pytest.raises(ppf.PPFError) as e:
        ppf.h5_dims(p, "nosuch")
    assert e.value.code == -3


def test_errors(tmp_path):
    p = str(tmp_path / "e.h5")
    ppf.h5_write(p, _fields((3, 3, 3)))
    with pytest.raises(ppf.PPFError) as e:
        ppf.h5_read(p, "/missing")
    assert e.value.code == -3
    with pytest.raises(ppf.PPFError) as e:
        ppf.h5_read(str(tmp_path / "none.h5"), "/etaS")
    assert e.value.code == -1
    bad = tmp_path / "bad.h5"
    bad.write_bytes(b"not an hdf5 file at all" * 10)
    with pytest.raises(ppf.PPFError) as e:
        ppf.h5_read(str(bad), "/etaS")
    assert e.value.code == -2
    # truncated: the data block is cut off
    raw = open(p, "rb").read()
    tr = tmp_path / "trunc.h5"
    tr.write_bytes(raw[: len(raw) - 100])
    for name in ("/etaS", "/c"):
        with pytest.raises(ppf.PPFError) as e:
            ppf.h5_read(str(tr), name)
        assert e.value.code == -1 and "truncated" in str(e.value)


def test_user_block_is_skipped(tmp_path):
    p = str(tmp_path / "u.h5")
    f = _fields((3, 4, 5), 9)
    ppf.h5_write(p, f)
    raw = open(p, "rb").read()
    # prepend a 512-byte user block; addresses are relative to the superblock
    ub = tmp_path / "ub.h5"
    ub.write_bytes(b"\0" * 512 + raw)
    assert np.array_equal(ppf.h5_read(str(ub), "etaS"), f["etaS"])


def test_metadata_dataset_round_trip(tmp_path):
    """The restart record: a (1, 1, n) float64 dataset next to the fields,
    found by name, leaving the fields as they were (contiguous and chunked)."""
    rng = np.random.default_rng(5)
    f = {k: rng.random((4, 5, 6)) for k in ("etaS", "etaL", "c")}
    rec = [123.0, 1.25e13, 7.0, 3.5e-9]
    for chunk in (None, (2, 5, 3)):
        p = str(tmp_path / f"m{chunk is None}.h5")
        ppf.h5_write(p, f, chunk=chunk, meta=("ppf_restart", rec))
        assert ppf.h5_dims(p, "ppf_restart") == (1, 1, 4)
        assert np.array_equal(ppf.h5_read(p, "ppf_restart").ravel(), rec)
        for k, v in f.items():
            assert np.array_equal(ppf.h5_read(p, k), v)


# ---- two independent implementations of the format: the product's and the oracle's ----

@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("shape,chunk", [((7, 9, 11), None), ((7, 9, 11), (2, 3, 4)), ((20, 33, 70), (5, 6, 7)),
                                         ((9, 9, 9), (1, 1, 1)), ((16, 16, 16), (8, 8, 8))])
def test_product_and_oracle_hdf5_read_each_other(tmp_path, dtype, shape, chunk):
    """Files written by the oracle's HDF5 code (oracle/hdf5_shim/h5ref.c,
    written separately from the format specification) read bit-exact with
    the product's reader and vice versa: contiguous, chunked with partial
    edge chunks, multi-level chunk B-trees (9^3 chunks of 1), float32."""
    import oracle
    f = _fields(shape, 11)
    po, pp = str(tmp_path / "o.h5"), str(tmp_path / "p.h5")
    oracle.h5_write(po, f, float32=dtype == "f32", chunk=chunk)
    ppf.h5_write(pp, f, dtype=dtype, chunk=chunk)
    for k, v in f.items():
        want = v.astype(np.float32).astype(np.float64) if dtype == "f32" else v
        assert np.array_equal(ppf.h5_read(po, k), want), k
        assert np.array_equal(oracle.h5_read(pp, k), want), k
        assert np.array_equal(oracle.h5_read(po, k), want), k


def test_oracle_reader_reads_data_written_by_libhdf5():
    """The MATLAB v7.3 fixture was written by libhdf5 (user block, base
    address 512, layout message version 2): the oracle's reader finds the
    rank-2 dataset and reads its values, x = 0:pi/4:2*pi."""
    import oracle
    p = _libhdf5_file()
    if p is None:
        pytest.skip("scipy test data not installed")
    assert oracle.h5_list(p)[0][:2] == ("testdouble", 2)
    x = oracle.h5_read_any(p, "testdouble")
    assert x.shape == (9, 1)
    assert np.allclose(x.ravel(), np.arange(9) * np.pi / 4, rtol=1e-15, atol=1e-15)


def test_reference_side_links_no_product_code():
    """The reference build's <hdf5.h> stand-in and the build recipe use the
    oracle's HDF5 code only."""
    here = os.path.dirname(os.path.abspath(__file__))
    shim = os.path.join(os.path.dirname(here), "oracle", "hdf5_shim")
    for fn in ("h5shim.c", "h5ref.c", "h5ref.h", "hdf5.h"):
        text = open(os.path.join(shim, fn)).read()
        assert "ppf_h5" not in text and "h5lite" not in text, fn
    recipe = open(os.path.join(os.path.dirname(here), "oracle", "build_ref.py")).read()
    assert "h5lite" not in recipe and "phasefield_coarsening_gb300" not in recipe


def _chunk_key_offsets(raw):
    """Offsets of the first chunk key's z origin in each raw-data B-tree node."""
    out, i = [], raw.find(b"TREE")
    while i >= 0:
        if raw[i + 4] == 1:
            out.append(i + 24 + 8)
        i = raw.find(b"TREE", i + 1)
    return out


@pytest.mark.parametrize("origin", [2 ** 63 + 4, 1, 2 ** 40])
def test_malformed_chunk_origin_is_rejected(tmp_path, origin):
    """A chunk origin outside the dataset or off the chunk grid is a format
    error, never a copy outside the output array."""
    p = str(tmp_path / "c.h5")
    ppf.h5_write(p, _fields((6, 6, 6), 3), chunk=(2, 3, 3))
    raw = bytearray(open(p, "rb").read())
    at = _chunk_key_offsets(bytes(raw))[0]
    raw[at:at + 8] = int(origin).to_bytes(8, "little")
    bad = tmp_path / "bad.h5"
    bad.write_bytes(bytes(raw))
    with pytest.raises(ppf.PPFError) as e:
        ppf.h5_read(str(bad), "etaS")
    assert e.value.code == -2

"""The files on either side of the path (libcvb, host only, no GPU): PETSc
binary vectors as VecView writes them, the restart set of
Ucont_P_Binary_Output / _Input (main.c:75-467), and grid.dat as MG_Initial
reads it (init.c:606-735).  The vector files are checked byte for byte
against PETSc's published binary layout, packed here independently with
struct, and the restart set against the files the reference's own
Ucont_P_Binary_Output writes (main.c compiled against the oracle's PETSc
shim, whose VecView / VecLoad follow the same published layout): the same
file names, block sizes and bytes, and the reference's Ucont_P_Binary_Input
reads the library's files to the same arrays.  Where the reference checkout
is absent (the GPU machine) the digests recorded from those reference-written
files stand in."""
import ctypes
import struct

import numpy as np
import pytest

from curvib_old_gb300 import _lib

CLASSID = 1211214


@pytest.fixture(scope="module")
def L():
    from curvib_old_gb300 import build
    build.build()
    return _lib.lib()


def _b(p):
    return str(p).encode()


def test_vector_file_layout_and_round_trip(L, tmp_path):
    v = np.random.default_rng(3).standard_normal(3 * 70)
    v[5] = -0.0
    v[6] = np.inf
    path = tmp_path / "vfield00007_0.dat"
    assert L.cvb_petsc_vec_write(_b(path), _lib.ptr(v), v.size, 3) == 0
    raw = path.read_bytes()
    assert raw == struct.pack(">ii", CLASSID, v.size) + struct.pack(f">{v.size}d", *v)
    assert (tmp_path / "vfield00007_0.dat.info").read_text() == "-vecload_block_size 3\n"
    n = ctypes.c_longlong()
    assert L.cvb_petsc_vec_size(_b(path), ctypes.byref(n)) == 0 and n.value == v.size
    back = np.empty_like(v)
    assert L.cvb_petsc_vec_read(_b(path), _lib.ptr(back), v.size) == 0
    assert back.tobytes() == v.tobytes()  # bit for bit, -0.0 and inf included


def test_vector_file_written_elsewhere_is_read(L, tmp_path):
    v = np.linspace(-1.0, 2.0, 11)
    path = tmp_path / "pfield00000_0.dat"
    path.write_bytes(struct.pack(">ii", CLASSID, v.size) + struct.pack(f">{v.size}d", *v))
    out = np.zeros_like(v)
    assert L.cvb_petsc_vec_read(_b(path), _lib.ptr(out), v.size) == 0
    assert np.array_equal(out, v)
    assert not (tmp_path / "pfield00000_0.dat.info").exists()


def test_vector_file_refusals(L, tmp_path):
    out = np.zeros(4)
    bad = tmp_path / "bad.dat"
    bad.write_bytes(struct.pack(">ii", 1211215, 4) + bytes(32))
    assert L.cvb_petsc_vec_read(_b(bad), _lib.ptr(out), 4) == 4
    short = tmp_path / "short.dat"
    short.write_bytes(struct.pack(">ii", CLASSID, 4) + bytes(24))
    assert L.cvb_petsc_vec_read(_b(short), _lib.ptr(out), 4) == 4
    good = tmp_path / "good.dat"
    good.write_bytes(struct.pack(">ii", CLASSID, 4) + bytes(32))
    assert L.cvb_petsc_vec_read(_b(good), _lib.ptr(out), 5) == 4  # length differs
    assert L.cvb_petsc_vec_read(_b(tmp_path / "missing.dat"), _lib.ptr(out), 4) == 4


def test_restart_set_names_and_round_trip(L, tmp_path):
    shape = (6, 5, 7)
    n = int(np.prod(shape))
    rng = np.random.default_rng(9)
    nvert, p = rng.random(shape), rng.standard_normal(shape)
    ucont, ucat = rng.standard_normal(shape + (3,)), rng.standard_normal(shape + (3,))
    assert L.cvb_restart_write(_b(tmp_path), 12, 0, n, _lib.ptr(nvert), _lib.ptr(ucont), _lib.ptr(ucat),
                               _lib.ptr(p)) == 0
    names = sorted(f.name for f in tmp_path.iterdir())
    assert names == ["nvfield00012_0.dat", "pfield00012_0.dat", "ufield00012_0.dat", "ufield00012_0.dat.info",
                     "vfield00012_0.dat", "vfield00012_0.dat.info"]
    u2, p2, nv2 = np.zeros_like(ucont), np.zeros_like(p), np.zeros_like(nvert)
    assert L.cvb_restart_read(_b(tmp_path), 12, 0, n, _lib.ptr(u2), _lib.ptr(p2), _lib.ptr(nv2)) == 0
    assert np.array_equal(u2, ucont) and np.array_equal(p2, p) and np.array_equal(nv2, nvert)
    assert L.cvb_restart_read(_b(tmp_path), 13, 0, n, _lib.ptr(u2), None, None) == 4  # no such step


def _grid_file(path, blocks, grid1d=False):
    lines = [str(len(blocks))]
    for nodes in blocks:
        KM, JM, IM = nodes.shape[:3]
        lines.append(f"{IM} {JM} {KM}")
        if grid1d:
            for i in range(IM):
                lines.append(f"{float(nodes[0, 0, i, 0])!r} 0.0 0.0")
            for j in range(JM):
                lines.append(f"0.0 {float(nodes[0, j, 0, 1])!r} 0.0")
            for k in range(KM):
                lines.append(f"0.0 0.0 {float(nodes[k, 0, 0, 2])!r}")
        else:
            for c in range(3):
                lines.extend(repr(float(x)) for x in nodes[..., c].ravel())
    path.write_text("\n".join(lines) + "\n")


def _read(L, path, block, grid1d, cl, ldim):
    im, jm, km = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert L.cvb_grid_dat_read(_b(path), block, grid1d, cl, ldim, ctypes.byref(im), ctypes.byref(jm),
                               ctypes.byref(km), None, 0) == 0
    out = np.zeros((km.value, jm.value, im.value, 3))
    assert L.cvb_grid_dat_read(_b(path), block, grid1d, cl, ldim, ctypes.byref(im), ctypes.byref(jm),
                               ctypes.byref(km), _lib.ptr(out), out.size) == 0
    return out


def test_grid_dat_blocks_and_scaling(L, tmp_path):
    from curvib_old_gb300 import workload as W
    a = W.box_nodes((6, 4, 5), (1.0, 2.0, 0.5), 2.0, True)
    b = W.box_nodes((3, 7, 4), (2.0, 1.0, 1.0), 1.5, True)
    path = tmp_path / "grid.dat"
    _grid_file(path, [a, b])
    assert np.array_equal(_read(L, path, 0, 0, 1.0, 1.0), a)
    cl, ldim = 0.3, 1.7
    assert np.array_equal(_read(L, path, 1, 0, cl, ldim), b / cl * ldim)
    im = ctypes.c_int()
    assert L.cvb_grid_dat_read(_b(path), 2, 0, 1.0, 1.0, ctypes.byref(im), ctypes.byref(im), ctypes.byref(im),
                               None, 0) == 4
    small = np.zeros(3)
    assert L.cvb_grid_dat_read(_b(path), 0, 0, 1.0, 1.0, ctypes.byref(im), ctypes.byref(im), ctypes.byref(im),
                               _lib.ptr(small), small.size) == 4


def test_grid_dat_one_dimensional_form(L, tmp_path):
    x, y, z = np.linspace(0, 1, 5), np.linspace(0, 2, 4) ** 1.5, np.linspace(-1, 1, 3)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    nodes = np.stack([X, Y, Z], axis=-1)
    path = tmp_path / "grid1d.dat"
    _grid_file(path, [nodes], grid1d=True)
    assert np.array_equal(_read(L, path, 0, 1, 1.0, 1.0), nodes)


def test_grid_dat_malformed(L, tmp_path):
    path = tmp_path / "grid.dat"
    path.write_text("1\n3 3 3\n0.0 1.0 oops\n")
    im = ctypes.c_int()
    out = np.zeros(81)
    assert L.cvb_grid_dat_read(_b(path), 0, 0, 1.0, 1.0, ctypes.byref(im), ctypes.byref(im), ctypes.byref(im),
                               _lib.ptr(out), out.size) == 4


@pytest.mark.parametrize("grid1d", [0, 1])
def test_grid_dat_matches_reference_mg_initial(L, tmp_path, grid1d):
    """The reference's own MG_Initial (init.c:296-1060, compiled against the
    oracle's PETSc shim) reads the same grid.dat to the same node coordinates,
    bit for bit, with the cl / L_dim scaling."""
    from oracle import oracle as O
    if not (O.REF_DIR / "init.c").exists():
        pytest.skip("reference checkout not present")
    from curvib_old_gb300 import workload as W
    ref = ctypes.CDLL(str(O.build_reference()))
    if grid1d:
        x, y, z = np.linspace(0, 1.3, 9), np.linspace(0, 2, 7) ** 1.5, np.linspace(-1, 1, 11)
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        nodes = np.stack([X, Y, Z], axis=-1)
    else:
        nodes = W.box_nodes((8, 6, 10), (1.0, 2.0, 0.5), 2.0, True)
    _grid_file(tmp_path / "grid.dat", [nodes], grid1d=bool(grid1d))
    (tmp_path / "bcs.dat").write_text("1 1 1 1 1 1\n")
    cl, ldim = 0.3, 1.7
    got = np.zeros(nodes.size)
    im, jm, km = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert ref.ref_mg_initial_nodes(_b(tmp_path), 2, grid1d, ctypes.c_double(cl), ctypes.c_double(ldim),
                                    ctypes.byref(im), ctypes.byref(jm), ctypes.byref(km),
                                    got.ctypes.data_as(ctypes.c_void_p), ctypes.c_longlong(got.size)) == 0
    assert (km.value, jm.value, im.value) == nodes.shape[:3]
    assert np.array_equal(_read(L, tmp_path / "grid.dat", 0, grid1d, cl, ldim).ravel(), got)


def _bcs(L, path, nblocks=1):
    bc = (ctypes.c_int * (6 * nblocks))()
    per = (ctypes.c_int * 3)()
    rc = L.cvb_bcs_dat_read(_b(path), nblocks, bc, per)
    return rc, list(bc), list(per)


def test_bcs_dat_read(L, tmp_path):
    """bcs.dat as MG_Initial reads it (init.c:474-490): six types per block,
    fscanf's %i (0x hexadecimal, 0 octal), and the periodic flags."""
    p = tmp_path / "bcs.dat"
    p.write_text("7 7 1 1 5 4\n")
    assert _bcs(L, p) == (0, [7, 7, 1, 1, 5, 4], [1, 0, 0])
    p.write_text("0x1 010 1 1 7 7\n1 1 7 7 1 1\n")
    assert _bcs(L, p, 2) == (0, [1, 8, 1, 1, 7, 7, 1, 1, 7, 7, 1, 1], [0, 1, 1])
    p.write_text("1 1 1 1 1\n")
    assert _bcs(L, p)[0] == _lib.CVB_BAD_INPUT
    assert _bcs(L, tmp_path / "missing.dat")[0] == _lib.CVB_BAD_INPUT


def test_bcs_dat_matches_reference_mg_initial(L, tmp_path):
    """The reference's own MG_Initial reads the same bcs.dat to the same
    boundary types and periodic flags."""
    from oracle import oracle as O
    if not (O.REF_DIR / "init.c").exists():
        pytest.skip("reference checkout not present")
    from curvib_old_gb300 import workload as W
    ref = ctypes.CDLL(str(O.build_reference()))
    nodes = W.box_nodes((8, 6, 10), (1.0, 2.0, 0.5), 2.0, True)
    _grid_file(tmp_path / "grid.dat", [nodes])
    (tmp_path / "bcs.dat").write_text("0x1 01 1 3 5 4\n")
    got = np.zeros(nodes.size)
    im, jm, km = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert ref.ref_mg_initial_nodes(_b(tmp_path), 2, 0, ctypes.c_double(1.0), ctypes.c_double(1.0), ctypes.byref(im),
                                    ctypes.byref(jm), ctypes.byref(km), got.ctypes.data_as(ctypes.c_void_p),
                                    ctypes.c_longlong(got.size)) == 0
    bc, per = (ctypes.c_int * 6)(), (ctypes.c_int * 3)()
    assert ref.ref_mg_initial_bctype(bc, per) == 0
    assert _bcs(L, tmp_path / "bcs.dat") == (0, list(bc), list(per))


def _restart_fields(shape, seed):
    rng = np.random.default_rng(seed)
    nvert = np.where(rng.random(shape) < 0.2, 3.0, 0.0)
    p = rng.standard_normal(shape)
    p[0, 0, 0] = -0.0
    return nvert, rng.standard_normal(shape + (3,)), rng.standard_normal(shape + (3,)), p


def test_restart_set_matches_reference_output(L, tmp_path):
    """The reference's Ucont_P_Binary_Output and cvb_restart_write produce the
    same files byte for byte; the reference's Ucont_P_Binary_Input reads the
    library's files to the arrays that were written."""
    from oracle import oracle as O
    import hashlib
    import json
    from pathlib import Path
    from cases import build
    c = build("box_sphere")
    shape = c["nvert"].shape
    nvert, ucont, ucat, p = _restart_fields(shape, 21)
    n = int(np.prod(shape))
    ours = tmp_path / "ours"
    ours.mkdir()
    assert L.cvb_restart_write(_b(ours), 37, 0, n, _lib.ptr(nvert), _lib.ptr(ucont), _lib.ptr(ucat),
                               _lib.ptr(p)) == 0
    got = {f.name: hashlib.sha256(f.read_bytes()).hexdigest()[:32] for f in sorted(ours.iterdir())}
    golden = json.loads((Path(__file__).parent / "golden" / "reference_digests.json").read_text())
    if (O.REF_DIR / "main.c").exists():
        R = O.Reference(c["nodes"], c["nl"], c["bctype"], c["semi"])
        theirs = tmp_path / "theirs"
        theirs.mkdir()
        R.restart_write(theirs, 37, 0, nvert, ucont, ucat, p)
        ref = {f.name: hashlib.sha256(f.read_bytes()).hexdigest()[:32] for f in sorted(theirs.iterdir())}
        assert got == ref
        assert ref == golden["restart"]
        uc2, p2, nv2 = R.restart_read(ours, 37, 0)
        assert uc2.tobytes() == ucont.tobytes() and p2.tobytes() == p.tobytes() and nv2.tobytes() == nvert.tobytes()
    else:
        assert got == golden["restart"]

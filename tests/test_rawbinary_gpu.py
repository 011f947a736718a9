"""Field snapshots in OpFlow's raw binary format (Utils::RawBinaryOStream / RawBinaryIStream,
src/Utils/Writers/RawBinaryStream.hpp:80-224).

Pinned to files the reference's own writer produced (tests/golden/rawbinary_ref.npz: the reference
driver compiles RawBinaryStream.hpp with its call to the removed CartesianField::evalSafeAt renamed
to evalAt): the engine writes the same fields byte for byte and reads the reference's files back into
the same values.  The layout is also checked field by field with an independent Python reader, and
the engine's reader by round trips and by its refusals of mismatched files.
"""
import os
import struct

import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from common import parse_cart
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

pytestmark = pytest.mark.gpu


def _fields(ctx, seed=51):
    mesh = cm.mesh_points([cm.stretched_points(7), cm.stretched_points(6, 2.0)])
    fc = cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_NEUM), (capi.BC_PERIODIC, capi.BC_PERIODIC)],
                       [(0.5, -1.0), (0.0, 0.0)], ext=1)
    fv = cm.field_desc(2, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC), (capi.BC_NEUM, capi.BC_DIRC)], [(0.25, -0.75), (0.0, 1.0)])
    out = []
    for name, fd, s in (("c", fc, seed), ("v", fv, seed + 1)):
        h = orc.HostField(mesh, fd)
        rng = h.assignable()
        j, i = np.meshgrid(np.arange(*rng[1]), np.arange(*rng[0]), indexing="ij")
        h.data[h.slices(rng)] = orc.u01(s, j.astype(np.uint64) * np.uint64(7) + i.astype(np.uint64))
        h.update_padding()
        f = api.CartesianField(mesh, fd, ctx, name)
        f.upload(h.data, update_padding=False)
        out.append(f)
    return mesh, out


def test_written_layout_follows_the_reference(ctx, tmp_path):
    mesh, (c, v) = _fields(ctx)
    os_ = api.RawBinaryOStream(str(tmp_path / "snap"))
    os_ << api.TimeStamp(0.25) << c << v
    os_ << api.TimeStamp(1.5) << c
    assert sorted(os.listdir(tmp_path)) == ["c_0.cart", "c_2.cart", "v_1.cart"]
    for fname, f, t in (("c_0.cart", c, 0.25), ("v_1.cart", v, 0.25), ("c_2.cart", c, 1.5)):
        rec = parse_cart(str(tmp_path / fname))
        assert rec["name"] == f.name and rec["dim"] == 2 and rec["nproc"] == 1 and rec["time"] == t
        for d in range(2):
            n = mesh.dims[d]
            assert rec["mesh_range"][d] == (0, n)
            assert np.array_equal(rec["coords"][d], np.asarray(mesh.x[d])[mesh.pad_width:mesh.pad_width + n])
            assert rec["accessible"][d] == tuple(f.info.accessible[d])
            assert rec["local"][d] == tuple(f.info.local[d])
        want = f.download()[f.index_slices([tuple(f.info.local[d]) for d in range(2)])].reshape(-1)
        assert np.array_equal(rec["values"], want)


def test_read_restores_the_field(ctx, tmp_path):
    mesh, (c, v) = _fields(ctx)
    os_ = api.RawBinaryOStream(str(tmp_path / "x"))
    os_ << api.TimeStamp(3.0) << c << v
    c2 = api.CartesianField(c.mesh, c.desc, ctx, "c")
    v2 = api.CartesianField(v.mesh, v.desc, ctx, "v")
    c2.assign(0.)
    v2.assign(0.)
    is_ = api.RawBinaryIStream(str(tmp_path / "x"))
    is_ >> c2
    assert is_.time == 3.0
    is_ >> v2
    assert np.array_equal(c2.download(), c.download())
    assert np.array_equal(v2.download(), v.download())


def test_mismatched_files_are_refused(ctx, tmp_path):
    mesh, (c, v) = _fields(ctx)
    api.RawBinaryOStream(str(tmp_path / "x")) << c
    other = api.CartesianField(cm.mesh_uniform([7, 6]), c.desc, ctx, "c")  # same shape, other coordinates
    with pytest.raises(capi.OpflowError) as e:
        api.RawBinaryIStream(str(tmp_path / "x")) >> other
    assert "coordinate" in str(e.value)
    wrong_loc = api.CartesianField(mesh, v.desc, ctx, "c")  # nodal field reading a cell-centred file
    with pytest.raises(capi.OpflowError):
        api.RawBinaryIStream(str(tmp_path / "x")) >> wrong_loc
    missing = api.CartesianField(mesh, c.desc, ctx, "nothere")
    with pytest.raises(capi.OpflowError):
        api.RawBinaryIStream(str(tmp_path / "x")) >> missing


def test_engine_writes_the_reference_files_byte_for_byte(ctx, tmp_path):
    meta, arr = cm.golden("rawbinary_ref")
    mesh, (c, v) = _fields(ctx, seed=int(meta["args"][1]))
    os_ = api.RawBinaryOStream(str(tmp_path / "snap"))
    os_ << api.TimeStamp(0.25) << c << v
    os_ << api.TimeStamp(1.5) << c
    for f in meta["files"]:
        mine = open(str(tmp_path / f), "rb").read()
        assert mine == arr["file__" + f[:-5]].tobytes(), f


def test_engine_reads_the_reference_files(ctx, tmp_path):
    meta, arr = cm.golden("rawbinary_ref")
    for f in meta["files"]:
        (tmp_path / f).write_bytes(arr["file__" + f[:-5]].tobytes())
    mesh, (c, v) = _fields(ctx, seed=int(meta["args"][1]))
    c2 = api.CartesianField(c.mesh, c.desc, ctx, "c")
    v2 = api.CartesianField(v.mesh, v.desc, ctx, "v")
    c2.assign(0.)
    v2.assign(0.)
    is_ = api.RawBinaryIStream(str(tmp_path / "snap"))
    is_ >> c2
    assert is_.time == 0.25
    is_ >> v2
    for g, ref in ((c2, c), (v2, v)):
        sl = g.index_slices([tuple(g.info.local[d]) for d in range(2)])
        assert np.array_equal(g.download()[sl], ref.download()[sl])

"""JSON graphs (ufo-core's format) and slice files, through the C ABI.

The parser and the file code are host C: these tests need no GPU, except the
last ones, which run a whole graph (read -> method -> write) and compare the
volumes with the oracle.
"""
import json
import os
import struct

import numpy as np
import pytest


def _graph(method="sirt", method_props=None, proj_props=None, read=None, write=None, edges=True, package="ir"):
    proj = {"plugin": "parallel-projector", "name": "proj", "package": "ir",
            "properties": {"model": "joseph", "is_forward": False, "step": 0.0523599}}
    if proj_props:
        proj["properties"].update(proj_props)
    props = {"projector": proj}
    props.update(method_props or {})
    nodes = [{"plugin": method, "name": "recon", "package": package, "properties": props}]
    if read is not None:
        nodes.insert(0, {"plugin": "read", "name": "in", "properties": read})
    if write is not None:
        nodes.append({"plugin": "write", "name": "out", "properties": write})
    doc = {"nodes": nodes}
    if edges:
        doc["edges"] = []
        if read is not None:
            doc["edges"].append({"from": {"name": "in"}, "to": {"name": "recon"}})
        if write is not None:
            doc["edges"].append({"from": {"name": "recon"}, "to": {"name": "out"}})
    return json.dumps(doc, indent=2)


def test_asdpocs_graph_with_nested_nodes(ufoir_lib):
    u = ufoir_lib
    text = _graph("asdpocs", {"num-iterations": 7, "beta_red": 0.99, "positive_constraint": False,
                              "df_minimizer": {"plugin": "sart", "package": "ir", "name": "inner",
                                               "properties": {"relaxation_factor": 0.3, "num-iterations": 12}}},
                  read={"path": "sino_*.tif"}, write={"filename": "vol%04i.tif"})
    g = u.graph_parse(text)
    assert g.method == u.METHOD_ASDPOCS
    assert g.asdpocs.num_iterations == 7 and g.asdpocs.beta_red == np.float32(0.99)
    assert g.asdpocs.positive_constraint == 0 and g.asdpocs.alpha == np.float32(0.2)   # default kept
    assert g.asdpocs.df_minimizer.num_iterations == 12
    assert g.asdpocs.df_minimizer.relaxation_factor == np.float32(0.3)
    assert g.projector.is_forward == 0 and g.projector.step == np.float32(0.0523599)
    assert g.projector.axis_position == -1.0 and g.projector.model == b"joseph"
    assert g.read_path == b"sino_*.tif" and g.write_filename == b"vol%04i.tif"
    j = u.graph_job_desc(g, 64, 60)
    assert j.method == u.METHOD_ASDPOCS and j.n_dets == 64 and j.n_angles == 60
    assert j.asdpocs.df_minimizer.num_iterations == 12 and j.step == g.projector.step


def test_dash_and_underscore_are_one_name(ufoir_lib):
    a = ufoir_lib.graph_parse(_graph("sart", {"num_iterations": 3, "relaxation-factor": 0.5}))
    b = ufoir_lib.graph_parse(_graph("sart", {"num-iterations": 3, "relaxation_factor": 0.5}))
    assert a.method == b.method == ufoir_lib.METHOD_SART
    assert a.sart.num_iterations == b.sart.num_iterations == 3
    assert a.sart.relaxation_factor == b.sart.relaxation_factor == np.float32(0.5)


def test_sbtv_and_extension_norm_mode(ufoir_lib):
    g = ufoir_lib.graph_parse(_graph("sbtv", {"lambda": 0.05, "mu": 1.0, "norm-mode": "compat"}))
    assert g.method == ufoir_lib.METHOD_SBTV and g.sbtv.mu == 1.0 and g.sbtv.norm_mode == ufoir_lib.NORM_COMPAT
    with pytest.raises(ufoir_lib.UfoirError) as e:
        ufoir_lib.graph_job_desc(g, 16, 16)
    assert e.value.status == ufoir_lib.ERR_UNSUPPORTED


@pytest.mark.parametrize("text,status,words", [
    (_graph("sirt", {"relaxation_factor": 1.5}), -1, "relaxation_factor"),
    (_graph("sirt", {"num-iterations": 0}), -1, "num-iterations"),
    (_graph("sirt", {"num-iterations": 2.5}), -1, "num-iterations"),
    (_graph("sirt", {"no-such-thing": 1}), -1, "no-such-thing"),
    (_graph("sirt", proj_props={"axis_position": -2.0}), -1, "axis_position"),
    (_graph("sirt", proj_props={"is_forward": 0}), -1, "is_forward"),
    (_graph("asdpocs", {"ng": 5000}), -1, "ng"),
    (_graph("fbp"), -4, "fbp"),
    (_graph("sirt", package="filters"), -4, "sirt"),
    (_graph("sirt", read={"path": "x.tif", "y-step": 2}), -4, "y-step"),
    (_graph("sirt", write={"filename": "a.tif", "bits": 16}), -1, "bits"),
    ('{"nodes": [{"plugin": "sirt", "package": "ir", "properties": {}}]}', -1, "projector"),
    ('{"nodes": []}', -1, "method"),
    ('{"nodes": [1, }', -10, "line 1"),
    ('{"nodes": [], "nodes": []}', -10, "duplicate"),
    ('{"nodes": [], "extra": 1}', -1, "extra"),
])
def test_invalid_graphs_are_refused_with_a_message(ufoir_lib, text, status, words):
    with pytest.raises(ufoir_lib.UfoirError) as e:
        ufoir_lib.graph_parse(text)
    assert e.value.status == status and words in str(e.value)


def test_edges_must_join_read_method_write(ufoir_lib):
    doc = json.loads(_graph("sirt", read={"path": "a.tif"}, write={"filename": "b.tif"}))
    doc["edges"] = [{"from": {"name": "in"}, "to": {"name": "out"}}]
    with pytest.raises(ufoir_lib.UfoirError):
        ufoir_lib.graph_parse(json.dumps(doc))
    doc["edges"] = [{"from": {"name": "in"}, "to": {"name": "recon"}}]      # write never fed
    with pytest.raises(ufoir_lib.UfoirError):
        ufoir_lib.graph_parse(json.dumps(doc))


def test_json_strings_numbers_and_escapes(ufoir_lib):
    # json.dumps escapes non-ASCII as \uXXXX (the emoji as a surrogate pair)
    text = _graph("sirt", read={"path": "déjà/\U0001F600/s.tif"}, write={"filename": "o\\x.tif"})
    text = text.replace("0.0523599", "5.23599e-2")
    g = ufoir_lib.graph_parse(text)
    assert g.read_path.decode("utf-8") == "déjà/\U0001F600/s.tif"
    assert g.write_filename == b"o\\x.tif"
    assert g.projector.step == np.float32(5.23599e-2)


def test_graph_load_from_file(ufoir_lib, tmp_path):
    p = tmp_path / "graph.json"
    p.write_text(_graph("sart", {"num-iterations": 4}))
    assert ufoir_lib.graph_load(str(p)).sart.num_iterations == 4
    with pytest.raises(ufoir_lib.UfoirError):
        ufoir_lib.graph_load(str(tmp_path / "missing.json"))


def test_tiff_round_trip_multi_page(ufoir_lib, tmp_path):
    rng = np.random.default_rng(4)
    a = rng.standard_normal((3, 17, 29)).astype(np.float32)
    a[0, 0, 0] = np.float32(-0.0)
    a[1, 2, 3] = np.float32(1e-41)          # subnormal survives
    f = str(tmp_path / "stack.tif")
    ufoir_lib.write_tiff(f, a)
    assert ufoir_lib.tiff_info(f) == (29, 17, 3)
    for k in range(3):
        b = ufoir_lib.read_tiff(f, k)
        assert b.tobytes() == a[k].tobytes()
    with pytest.raises(ufoir_lib.UfoirError):
        ufoir_lib.read_tiff(f, 3)


def _tiff_bytes_be_uint16(img, rows_per_strip):
    """A big-endian, multi-strip, uint16 TIFF built by hand."""
    h, w = img.shape
    strips = [img[r:r + rows_per_strip] for r in range(0, h, rows_per_strip)]
    data = [s.astype(">u2").tobytes() for s in strips]
    n_tags = 9
    ifd_at = 8
    after_ifd = ifd_at + 2 + 12 * n_tags + 4
    offsets_at = after_ifd
    counts_at = offsets_at + 4 * len(strips)
    data_at = counts_at + 4 * len(strips)
    offs, pos = [], data_at
    for d in data:
        offs.append(pos)
        pos += len(d)
    out = b"MM" + struct.pack(">HI", 42, ifd_at)
    tags = [(256, 4, 1, w), (257, 4, 1, h), (258, 3, 1, 16), (259, 3, 1, 1), (262, 3, 1, 1),
            (273, 4, len(strips), offsets_at), (277, 3, 1, 1), (278, 4, 1, rows_per_strip),
            (279, 4, len(strips), counts_at)]
    out += struct.pack(">H", n_tags)
    for tag, typ, cnt, val in tags:
        if typ == 3 and cnt == 1:
            out += struct.pack(">HHIHH", tag, typ, cnt, val, 0)
        else:
            out += struct.pack(">HHII", tag, typ, cnt, val)
    out += struct.pack(">I", 0)
    out += struct.pack(">" + "I" * len(offs), *offs)
    out += struct.pack(">" + "I" * len(data), *[len(d) for d in data])
    return out + b"".join(data)


def test_tiff_big_endian_uint16_strips(ufoir_lib, tmp_path):
    img = (np.arange(7 * 11, dtype=np.uint32).reshape(7, 11) * 797 % 65536).astype(np.uint16)
    f = tmp_path / "be.tif"
    f.write_bytes(_tiff_bytes_be_uint16(img, 3))
    assert ufoir_lib.tiff_info(str(f)) == (11, 7, 1)
    assert np.array_equal(ufoir_lib.read_tiff(str(f)), img.astype(np.float32))


def test_tiff_rejects_what_it_cannot_read(ufoir_lib, tmp_path):
    f = tmp_path / "x.tif"
    f.write_bytes(b"GIF89a" + b"\0" * 32)
    with pytest.raises(ufoir_lib.UfoirError) as e:
        ufoir_lib.tiff_info(str(f))
    assert e.value.status == ufoir_lib.ERR_IO and "not a TIFF" in str(e.value)
    f.write_bytes(b"II" + struct.pack("<HI", 42, 4000))              # IFD beyond the end
    with pytest.raises(ufoir_lib.UfoirError):
        ufoir_lib.tiff_info(str(f))


def test_raw_round_trip(ufoir_lib, tmp_path):
    a = np.random.default_rng(1).random((5, 13), dtype=np.float32)
    f = str(tmp_path / "a.raw")
    ufoir_lib.write_raw(f, a)
    assert np.array_equal(ufoir_lib.read_raw(f, (5, 13)), a)
    assert np.array_equal(ufoir_lib.read_raw(f, (13,), offset=4 * 13 * 2), a[2])
    with pytest.raises(ufoir_lib.UfoirError):
        ufoir_lib.read_raw(f, (6, 13))


# ------------------------------------------------------------------ on a GPU

@pytest.mark.gpu
def test_graph_run_sirt_tiff_per_slice_output(ufoir_lib, gpu_ctx, oracle, tmp_path):
    u = ufoir_lib
    n, na, iters = 40, 36, 4
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(11)
    sinos = np.stack([oracle.forward(oracle.projector(n, na, step), rng.random((n, n), dtype=np.float32))
                      for _ in range(3)])
    for i in range(3):
        u.write_tiff(str(tmp_path / f"sino_{i:02d}.tif"), sinos[i])
    text = _graph("sirt", {"num-iterations": iters}, proj_props={"step": float(step)},
                  read={"path": str(tmp_path / "sino_*.tif")}, write={"filename": str(tmp_path / "vol%03i.tif")})
    g = u.graph_parse(text)
    assert u.graph_run(gpu_ctx, g) == 3
    for i in range(3):
        got = u.read_tiff(str(tmp_path / f"vol{i:03d}.tif"))
        want = oracle.sirt(oracle.projector(n, na, step), sinos[i], iters, 0.25)
        assert np.array_equal(got, want)


@pytest.mark.gpu
def test_graph_run_asdpocs_raw_in_multipage_out(ufoir_lib, gpu_ctx, oracle, tmp_path):
    u = ufoir_lib
    n, na = 32, 30
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(12)
    sinos = np.stack([oracle.forward(oracle.projector(n, na, step), rng.random((n, n), dtype=np.float32))
                      for _ in range(2)])
    u.write_raw(str(tmp_path / "sinos.raw"), sinos)
    props = {"num-iterations": 2, "norm-mode": "compat",
             "df_minimizer": {"plugin": "sart", "package": "ir", "properties": {"num-iterations": 2}}}
    text = _graph("asdpocs", props, proj_props={"step": float(step)},
                  read={"path": str(tmp_path / "sinos.raw"), "raw-width": n, "raw-height": na},
                  write={"filename": str(tmp_path / "vol.tif")})
    assert u.graph_run(gpu_ctx, u.graph_parse(text)) == 2
    p = u.ParallelProjector(gpu_ctx, step=float(step), is_forward=0)
    want = u.asdpocs(p, sinos, num_iterations=2, norm_mode=u.NORM_COMPAT, df_minimizer=dict(num_iterations=2))
    p.close()
    assert u.tiff_info(str(tmp_path / "vol.tif")) == (n, n, 2)
    for i in range(2):
        assert np.array_equal(u.read_tiff(str(tmp_path / "vol.tif"), i), want[i])


@pytest.mark.gpu
def test_graph_run_refuses_a_bad_counter(ufoir_lib, gpu_ctx, tmp_path):
    u = ufoir_lib
    u.write_tiff(str(tmp_path / "s.tif"), np.zeros((12, 16), np.float32))
    text = _graph("sirt", {"num-iterations": 1}, proj_props={"step": 0.26},
                  read={"path": str(tmp_path / "s.tif")}, write={"filename": str(tmp_path / "v%s.tif")})
    with pytest.raises(u.UfoirError) as e:
        u.graph_run(gpu_ctx, u.graph_parse(text))
    assert e.value.status == u.ERR_INVALID and "counter" in str(e.value)

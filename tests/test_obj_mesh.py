"""OBJ cloth ingest (cloth_mesh_from_obj): the reference's cBaseCloth OBJ
branch over cObjUtil::LoadObj / BuildEdge.  The golden OBJ cases
(obj_irregular, obj_relocated) pin the loader bit for bit against the
reference itself; these cases cover the OBJ forms and refusals around them."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden


@pytest.fixture(scope="module")
def load(built):
    from acousticsim_gb300 import load_obj_mesh
    return load_obj_mesh


def _write(tmp_path, text, name="m.obj"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_golden_obj_matches_reference(load):
    for case in ("obj_irregular", "obj_relocated"):
        g, conf = load_golden(case)
        m = load(conf["cloth_obj_path"], conf["cloth_obj_translation"],
                 conf["enable_relocate_obj"])
        assert np.array_equal(m["pos"], g["topo_pos"])
        assert np.array_equal(m["uv"], g["topo_uv"])
        assert np.array_equal(m["tris"], g["topo_tris"])
        assert np.array_equal(m["edges"], g["topo_edges"][:, :4])
        # widths the regular grid never reaches
        assert (g["topo_ell"] >= 0).sum(1).max() > 13


def test_quad_split_follows_shorter_diagonal(load, tmp_path):
    # diagonal 0-2 shorter: [0 1 2] [0 2 3]; diagonal 1-3 shorter: [0 1 3] [1 2 3]
    a = _write(tmp_path, "v 0 0 0\nv 1 0 0\nv 0.8 1 0\nv 0 1 0\nf 1 2 3 4\n", "a.obj")
    b = _write(tmp_path, "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0.3 1 0\nf 1 2 3 4\n", "b.obj")
    assert load(a)["tris"].tolist() == [[0, 1, 2], [0, 2, 3]]
    assert load(b)["tris"].tolist() == [[0, 1, 3], [1, 2, 3]]


def test_index_forms_and_uv(load, tmp_path):
    text = ("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\n"
            "vt 0.0 0.0\nvt 0.3 0.0\nvt 0.0 0.3\nvt 0.3 0.3\nvn 0 0 1\n"
            "f 1/1/1 2/2/1 3/3/1\n"      # v/vt/vn
            "f -3/-3 -1/-1 -2/-2\n")     # negative (relative) v/vt
    m = load(_write(tmp_path, text), (0.0, 0.0, 0.0), False)
    assert m["tris"].tolist() == [[0, 1, 2], [1, 3, 2]]
    # y + 0.2; uv * 10/3 in float
    assert np.allclose(m["pos"][:, 1], [0.2, 0.2, 1.2, 1.2])
    s = np.float32(10 / 3.0)
    assert np.array_equal(m["uv"], np.array([[0, 0], [0.3, 0], [0, 0.3], [0.3, 0.3]],
                                            np.float32) * s)
    # edges: ascending vertex pairs, first and second triangle
    assert m["edges"].tolist() == [[0, 1, 0, -1], [0, 2, 0, -1], [1, 2, 0, 1], [1, 3, 1, -1],
                                   [2, 3, 1, -1]]
    # v//vn form, translation
    m2 = load(_write(tmp_path, "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1//1 2//1 3//1\n", "c.obj"),
              (1.0, 2.0, 3.0), False)
    assert np.allclose(m2["pos"][0], [1.0, 2.2, 3.0])
    assert np.all(m2["uv"] == 0)


def test_relocation(load, tmp_path):
    text = "v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1.005 0\nf 1 2 3\nf 2 4 3\n"
    m = load(_write(tmp_path, text), (0.5, 0.0, 0.25), True)
    assert abs(m["pos"][:, 1].max() - 0.27) < 1e-7
    # x, z centred on the vertices within 1 cm of the top (vertices 2 and 3)
    assert abs(m["pos"][2:, 0].mean()) < 1e-12
    assert np.allclose(m["pos"][:, 2], 0.0)


@pytest.mark.parametrize("text, what", [
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nv 2 2 0\nf 1 2 3 4 5\n", "faces of 5"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 5 5 5\nf 1 2 3\nf 1 2 4\nf 2 1 5\n", "bad face index"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nv 9 9 9\nf 1 2 3\nf 2 4 3\nf 1 3 5\nf 1 2 5\n"
     "f 2 1 4\n", "more than two"),
    ("v 0 0 0\n", "no faces"),
])
def test_refusals(load, tmp_path, text, what):
    from acousticsim_gb300 import ClothError
    with pytest.raises(ClothError) as e:
        load(_write(tmp_path, text))
    assert what in str(e.value)


def test_missing_file(load):
    from acousticsim_gb300 import ClothError
    with pytest.raises(ClothError):
        load("/nonexistent/cloth.obj")

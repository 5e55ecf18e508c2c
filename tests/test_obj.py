"""The OBJ loader (rt_obj_counts / rt_obj_load, host code): round trips of the
seeded scenes, the statement forms a mesh exporter writes, and rejection of
malformed files."""
from __future__ import annotations

import numpy as np
import pytest


def test_box_scene_round_trip(rtlib, tmp_path):
    import rtcore.scenes as S
    v, i, tm, m = S.box(S.SEED_BASE + 3, 3, 4)
    path = tmp_path / "box.obj"
    S.write_obj(path, v, i, tm)
    lv, li, ltm, nm = S.load_obj(path)
    assert lv.tobytes() == v.tobytes() and li.tobytes() == i.tobytes()
    # material indices are numbered by first use, which is the scene's order
    assert ltm.tobytes() == tm.tobytes() and nm == len(np.unique(tm))


def test_soup_round_trip(rtlib, tmp_path):
    import rtcore.scenes as S
    v, i = S.soup(S.SEED_BASE + 2, 5000)
    path = tmp_path / "soup.obj"
    S.write_obj(path, v, i)
    lv, li, ltm, nm = S.load_obj(path)
    assert lv.tobytes() == v.tobytes() and li.tobytes() == i.tobytes()
    assert nm == 1 and (ltm == 0).all()


def test_statement_forms(rtlib, tmp_path):
    import rtcore.scenes as S
    text = "\r\n".join([
        "# exported mesh", "mtllib scene.mtl", "o thing", "g group1", "s off",
        "v 0 0 0", "v 1 0 0", "v 1 1 0", "v 0 1 0", "v\t0.5\t2\t-1e-3   1.0",
        "vt 0 0", "vt 1 0", "vn 0 0 1",
        "f 1 2 3",                        # before any usemtl: the unnamed material
        "usemtl red",
        "f 1/1 2/2 3/1 4/2",              # quad -> two triangles
        "usemtl green  stripes",          # names may contain blanks
        "f -5//1 -4//1 -3//1 -2//1 -1//1",  # pentagon with negative references -> three
        "usemtl red",
        "f +4/1/1 3/2/1 5/1/1  # trailing comment",
        "l 1 2", "p 3", "",
    ]) + "\r\n"
    path = tmp_path / "forms.obj"
    path.write_bytes(text.encode())
    v, i, tm, nm = S.load_obj(path)
    assert v.shape == (5, 3) and tuple(v[4]) == (0.5, 2.0, np.float32(-1e-3))
    assert i.tolist() == [[0, 1, 2], [0, 1, 2], [0, 2, 3], [0, 1, 2], [0, 2, 3], [0, 3, 4], [3, 2, 4]]
    assert tm.tolist() == [0, 1, 1, 2, 2, 2, 1] and nm == 3


@pytest.mark.parametrize("body", [
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n",      # beyond the last vertex
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n",      # zero is not an index
    "v 0 0 0\nv 1 0 0\nf -3 1 2\n",              # relative reference before the first vertex
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2\n",        # fewer than three references
    "v 0 0 x\n",                                 # malformed number
    "v 0 0\n",                                   # missing coordinate
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3.5\n",    # fractional index
])
def test_malformed_files_are_rejected(rtlib, tmp_path, body):
    import rtcore
    import rtcore.scenes as S
    path = tmp_path / "bad.obj"
    path.write_text(body)
    with pytest.raises(rtcore.RtError) as e:
        S.load_obj(path)
    assert e.value.code == rtcore.RT_ERR_INVALID_ARG


def test_missing_file(rtlib, tmp_path):
    import rtcore
    import rtcore.scenes as S
    with pytest.raises(rtcore.RtError):
        S.load_obj(tmp_path / "nope.obj")
    v, i, tm, nm = (None,) * 4
    empty = tmp_path / "empty.obj"
    empty.write_text("# nothing\n")
    v, i, tm, nm = S.load_obj(empty)
    assert v.shape == (0, 3) and i.shape == (0, 3) and nm == 0

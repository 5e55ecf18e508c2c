"""The path tracer's command-line renderer (python -m rtcore.pt): the image
it writes equals the oracle's rendering of the same samples bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _read_pfm(path):
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = map(int, f.readline().split())
        assert float(f.readline()) < 0  # little-endian
        data = np.frombuffer(f.read(), np.float32)
    return data.reshape(h, w, 3)[::-1]  # PFM stores the bottom row first


def test_pt_cli_image_equals_oracle(ctx, orc, tmp_path, capsys):
    import json
    import rtcore.scenes as S
    from rtcore import pt
    w, h, spp = 64, 48, 2
    out = tmp_path / "box.pfm"
    assert pt.main(["--spheres", "3", "--freq", "6", "--width", str(w), "--height", str(h), "--spp", str(spp),
                    "--calls", "1", "--pfm", str(out), "--ppm", str(tmp_path / "box.ppm")]) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["resolution"] == [w, h] and line["ms_per_spp"] > 0
    img = _read_pfm(out)
    v, i, tm, m = S.box(S.SEED_BASE + 3, 3, 6)
    ob, _ = orc.build_blas([(v, i, None)])
    # one warm-up call and one timed call of spp samples each: 2 * spp samples
    acc = orc.path_trace(ob, tm, m, S.emissive_lights(v, i, tm, m), S.BOX_CAMERA, w, h, 2 * spp, 8, 3,
                         S.SEED_BASE + 3, 1e-4)
    want = (acc / np.maximum(acc[..., 3:4], 1.0))[..., :3].astype(np.float32)
    assert img.tobytes() == np.ascontiguousarray(want).tobytes()
    assert (tmp_path / "box.ppm").read_bytes().startswith(b"P6\n64 48\n255\n")

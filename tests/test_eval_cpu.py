"""save_keypoints (utils.cpp:97-152): the Mikolajczyk text format, written
by the library's host code, against the same format produced here."""
import numpy as np

import akaze_gb300 as akz


def _expected(kp, desc):
    lines = [str(desc.shape[1] if desc is not None else 1), str(len(kp))]
    for i in range(len(kp)):
        sc = np.float32(kp["size"][i]) * np.float32(kp["size"][i])
        r = 1.0 / float(sc)
        row = "%g %g %g %g %g" % (float(kp["x"][i]), float(kp["y"][i]), r, 0.0, r)
        if desc is not None:
            row += "".join(" %d" % v for v in desc[i])
        lines.append(row)
    return "\n".join(lines) + "\n"


def test_save_keypoints_format(tmp_path):
    rng = np.random.default_rng(0)
    kp = np.zeros(5, akz.KEYPOINT_DTYPE)
    kp["x"] = rng.uniform(0, 1920, 5).astype(np.float32)
    kp["y"] = rng.uniform(0, 1080, 5).astype(np.float32)
    kp["size"] = rng.uniform(4, 60, 5).astype(np.float32)
    desc = rng.integers(0, 256, (5, 61)).astype(np.uint8)
    p1, p2 = tmp_path / "with.txt", tmp_path / "without.txt"
    akz.save_keypoints(p1, kp, desc)
    akz.save_keypoints(p2, kp)
    assert p1.read_text() == _expected(kp, desc)
    assert p2.read_text() == _expected(kp, None)

"""Shared definitions of the golden fixtures (scene generators, inputs) for the tests."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)

from make_goldens import (SCENES, HALTON_RES, BSDF_PARAMS, SAMPLER_CASES, bsdf_inputs, bsdf_kind, ray_set,  # noqa: E402,F401
                          anyhit_inputs, hdr_images, sampler_scene)


def read_rgbe(data: bytes):
    """Decode a Radiance file (header, "-Y H +X W", flat or run-length scanlines) to (H, W, 4) uint8."""
    import numpy as np
    end = data.index(b"\n\n") + 2
    line_end = data.index(b"\n", end)
    _, h, _, w = data[end:line_end].split()
    h, w = int(h), int(w)
    pos = line_end + 1
    out = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if 8 <= w <= 32767 and data[pos] == 2 and data[pos + 1] == 2:
            assert (data[pos + 2] << 8 | data[pos + 3]) == w
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = data[pos]
                    if n > 128:
                        out[y, x:x + n - 128, c] = data[pos + 1]
                        x += n - 128
                        pos += 2
                    else:
                        assert n > 0
                        out[y, x:x + n, c] = np.frombuffer(data[pos + 1:pos + 1 + n], np.uint8)
                        x += n
                        pos += 1 + n
                assert x == w
        else:
            out[y] = np.frombuffer(data[pos:pos + 4 * w], np.uint8).reshape(w, 4)
            pos += 4 * w
    assert pos == len(data)
    return out

"""Shared definitions of the golden fixtures (scene generators, inputs) for the tests."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)

from make_goldens import SCENES, HALTON_RES, BSDF_PARAMS, bsdf_inputs, bsdf_kind, ray_set, anyhit_inputs  # noqa: E402,F401

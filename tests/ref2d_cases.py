"""Shared description of the reference-pinned 2D parity cases (tests/golden)."""
import ast

from metallic_glasses_gb300 import api, configs

CASES = ["ref2d_64_tension_s123", "ref2d_32_shear_s7", "ref2d_32_tension_nosoft_s5", "ref2d_32_shear_stop_s7"]


def params_for(g):
    ov = ast.literal_eval(str(g["overrides"]))
    loading = api.LOAD_SHEAR if str(g["loading"]) == "SHEAR" else api.LOAD_TENSION
    return configs.ref2d(int(g["nx"]), int(g["ny"]), loading=loading, **ov)

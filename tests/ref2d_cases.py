"""Shared description of the reference-pinned 2D parity cases (tests/golden)."""
import ast

import numpy as np

from metallic_glasses_gb300 import api, configs

CASES = ["ref2d_64_tension_s123", "ref2d_32_shear_s7", "ref2d_32_tension_nosoft_s5", "ref2d_32_shear_stop_s7",
         "ref2d_32x48_tension_s51"]


MRO_CASES = ["ref2d_32_mro_s11", "ref2d_32_mrofile_s13"]

# the reference built with each of the other softening-direction schemes
SF_CASES = ["ref2d_32_sf_linear_fwd_s21", "ref2d_32_sf_linear_bwd_s22", "ref2d_32_sf_even_s23",
            "ref2d_32_sf_cubic_fwd_s24", "ref2d_32_sf_gauss_fwd_s25"]

# the reference built with NO_SUBTRACT_ERROR, under TENSION and SHEAR
SWITCH_CASES = ["ref2d_32_tension_nse_s32", "ref2d_32_shear_nse_s33"]

# crystal-like sites with the reference built without NO_SF_XTAL_MRO
MRO_SWITCH_CASES = ["ref2d_32_mro_xsfoff_s11"]

# the reference built with a high-temperature material branch of Init()
MATERIAL_CASES = ["ref2d_32_vit1_s41", "ref2d_32_pdnip_s42"]


def params_for(g, material=None, **kw):
    """The engine parameters of fixture g (its input overrides, loading and
    switches); material "LOW_T" keeps the input file's derivation in place of
    the fixture's high-temperature branch."""
    ov = ast.literal_eval(str(g["overrides"]))
    loading = api.LOAD_SHEAR if str(g["loading"]) == "SHEAR" else api.LOAD_TENSION
    structure = str(g["structure"]) if "structure" in g.files else None
    p = configs.ref2d(int(g["nx"]), int(g["ny"]), loading=loading, mro_structure=structure, **kw, **ov)
    if "sf" in g.files:
        p.sf_scheme = int(g["sf"])
    if "nse" in g.files:
        p.no_subtract_error = int(g["nse"])
    if "xsf" in g.files:
        p.no_sf_xtal_mro = int(g["xsf"])
    material = material or (str(g["material"]) if "material" in g.files else "LOW_T")
    if material != "LOW_T":
        configs.high_t_material(p, material)
    return p


def check_mro_state(m, g, exact=True):
    """The crystal-like sites of an MRO fixture: the map and angles, their
    mode eigenstrains (drawn at the start and kept) and their barriers at the
    end (new ones drawn at each of their transformations)."""
    assert np.array_equal(m.field(api.FIELD_MRO, 0).astype(np.int8), g["mro"])
    assert np.array_equal(m.field(api.FIELD_MRO, 1), g["theta"])
    sel = np.nonzero(g["mro"])[0]
    deps = np.stack([m.field(api.FIELD_DEPS, k) for k in range(60)]).reshape(20, 3, -1)[:, :, sel]
    q0 = np.stack([m.field(api.FIELD_DF, k) for k in range(20)])[:, sel]
    if exact:
        assert np.array_equal(deps, g["deps_mro"])
        assert np.array_equal(q0, g["q0_mro"])
    else:
        assert np.abs(deps - g["deps_mro"]).max() <= 1e-15
        assert np.abs(q0 - g["q0_mro"]).max() <= 1e-14

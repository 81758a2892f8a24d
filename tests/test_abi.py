"""The C-ABI library loads without a GPU, exports every symbol include/obgc.h declares, and the
ctypes mirror matches the C struct layouts (no device work here)."""
import ctypes as C
import os
import re

import pytest

from obgc import _abi as A

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "obgc.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(obgc_[a-z0-9_]+)\s*\(", text)))


def test_library_loads_and_version():
    lib = A.load()
    assert lib.obgc_abi_version() == 2


def test_every_declared_symbol_is_exported():
    lib = A.load()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(A.EXPORTED) <= set(names)


@pytest.mark.parametrize("which,struct,fields", [
    (0, A.NPDParams, ["nitrification_rate", "phytoplankton_sinking_speed", "nitrification_oxygen_nitrogen_ratio"]),
    (1, A.TwoBandParams, ["chlorophyll_red_exponent", "pigment_ratio", "phytoplankton_chlorophyll_ratio"]),
    (2, A.Surface, ["value", "field", None]),
    (3, A.Grid, ["Lx", "stride_j", "stride_k"]),
    (4, A.CarbonOptions, ["density_value", "atol", "saturation_mineral"]),
    (5, A.ModelDesc, ["surface", "grid", "passive_tendency_of"]),
    (6, A.Fields, ["passive", "u", "G"]),
    (7, A.ColumnSpec, ["dz", "pulse_step", "salinity"]),
    (8, A.ColumnsDesc, ["light", "arena_cells", "gas"]),
    (9, A.PiscesParams, ["micro", "doc_aggregation", "open_bottom"]),
    (10, A.PiscesPhyto, ["exudated_fraction", "base_growth_rate", "silicate_half_saturation_parameter"]),
    (11, A.PiscesField, ["value", "data", None]),
    (12, A.GasExchange, ["wind_field", "o2_solubility", "carbon"]),
    (13, A.BoxDrivers, ["n_prescribed", "prescribed", "forcing"]),
])
def test_struct_layouts(which, struct, fields):
    lib = A.load()
    out = (C.c_int64 * 4)()
    assert lib.obgc_struct_layout(which, out, 4) == 0
    assert out[0] == C.sizeof(struct)
    for q, f in enumerate(fields):
        if f is not None:
            assert out[q + 1] == getattr(struct, f).offset, f


def test_bad_arguments_return_status_not_crash():
    lib = A.load()
    assert lib.obgc_npd_preset(7, C.byref(A.NPDParams())) == 1
    assert lib.obgc_npd_preset(0, None) == 1
    assert lib.obgc_npd_required_tracers(None, None, 0) < 0
    assert "preset" in lib.obgc_last_error_message().decode()


def test_no_device_is_reported():
    # In a container without a GPU, building a context fails with a status, not a crash.
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = A.load()
    d = A.ModelDesc()
    lib.obgc_npd_preset(0, C.byref(d.npd))
    d.grid.Nx = d.grid.Ny = d.grid.Nz = 4
    d.grid.Lx = d.grid.Ly = d.grid.Lz = 1.0
    d.grid.stride_j, d.grid.stride_k = 4, 16
    ctx = C.c_void_p()
    rc = lib.obgc_create(C.byref(d), C.byref(ctx))
    assert rc in (2, 7) and not ctx.value


def test_new_entry_points_reject_bad_arguments_without_a_device():
    # argument checks run before any device work, so they answer on a machine without a GPU
    lib = A.load()
    g = A.GasExchange()
    assert lib.obgc_gas_exchange_defaults(A.GAS_CO2, C.byref(g)) == 0
    assert lib.obgc_set_gas_exchange_on(None, A.NAME_INDEX["DIC"], C.byref(g), A.NAME_INDEX["DIC"], A.NAME_INDEX["Alk"]) == 1
    assert lib.obgc_set_forcing(None, A.NAME_INDEX["Alk"], None, 0.0, 1.0) == 1
    assert lib.obgc_set_vertical_time_discretization(None, A.VERTICALLY_IMPLICIT) == 1
    p = A.NPDParams()
    assert lib.obgc_npd_preset(A.PRESET_NPZD, C.byref(p)) == 0
    d = A.BoxDrivers()
    d.n_prescribed = A.BOX_MAX_DRIVERS + 1
    assert lib.obgc_box_run_drivers(C.byref(p), None, 1, C.c_void_p(1), C.byref(d), 0.0, 1.0, 1, 0, None,
                                    A.PREC_F64, None) == 1
    d.n_prescribed = 1
    d.prescribed_names[0] = A.NUM_NAMED                 # not a tracer name
    d.prescribed[0] = 1
    assert lib.obgc_box_run_drivers(C.byref(p), None, 1, C.c_void_p(1), C.byref(d), 0.0, 1.0, 1, 0, None,
                                    A.PREC_F64, None) == 1
    assert "prescribed" in lib.obgc_last_error_message().decode()


def test_step_status_entry_points_reject_a_null_context():
    lib = A.load()
    flags = C.c_int32(-1)
    assert lib.obgc_step_status(None, C.byref(flags)) == 1
    assert lib.obgc_set_status_check(None, 1) == 1

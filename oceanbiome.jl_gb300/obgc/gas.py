"""Air-sea gas exchange (src/Models/GasExchange): CarbonDioxideGasExchangeBoundaryCondition and
OxygenGasExchangeBoundaryCondition as flux models of the surface face, positive out of the ocean."""
import ctypes as C

from . import _abi as A


class CarbonDioxideConcentration:
    """CarbonDioxideConcentration(; DIC = :DIC, Alk = :Alk) (carbon_dioxide_concentration.jl:13-60):
    the tracers whose surface values give the water's pCO2, e.g. DIC = "DIC2", Alk = "Alk2" for the
    second replicate of CarbonateSystem(2)."""

    def __init__(self, DIC="DIC", Alk="Alk", carbon_chemistry=None):
        self.DIC, self.Alk, self.carbon_chemistry = DIC, Alk, carbon_chemistry


class GasExchange:
    """GasExchange(gas; wind_speed, air_concentration, transfer velocity / Schmidt / solubility
    coefficients): wind_speed and air_concentration are numbers or (Ny, Nx) device tensors.
    water_concentration: a CarbonDioxideConcentration (CO2; default DIC and Alk)."""

    def __init__(self, gas, wind_speed=None, air_concentration=None, k660=None, schmidt=None, o2_solubility=None,
                 carbon_chemistry=None, water_concentration=None):
        self.gas = gas
        if water_concentration is not None and gas != A.GAS_CO2:
            raise ValueError("water_concentration: the O2 condition reads its own tracer")
        self.water_concentration = water_concentration or (CarbonDioxideConcentration() if gas == A.GAS_CO2 else None)
        if carbon_chemistry is None and self.water_concentration is not None:
            carbon_chemistry = self.water_concentration.carbon_chemistry
        self.params = A.GasExchange()
        A.check(A.load().obgc_gas_exchange_defaults(gas, C.byref(self.params)), "obgc_gas_exchange_defaults")
        self._keep = []
        if carbon_chemistry is not None:
            self.params.carbon = carbon_chemistry.options
            self.params.carbon.output = A.OUT_PCO2
        for name, val in (("k660", k660), ("schmidt", schmidt), ("o2_solubility", o2_solubility)):
            if val is not None:
                arr = getattr(self.params, name)
                if len(val) > len(arr):
                    raise ValueError(f"{name}: at most {len(arr)} coefficients")
                for q in range(len(arr)):
                    arr[q] = float(val[q]) if q < len(val) else 0.0
        self._set("wind_speed", "wind_field", wind_speed)
        self._set("air_concentration", "air_field", air_concentration)

    def _set(self, value_name, field_name, x):
        if x is None:
            return
        if isinstance(x, (int, float)):
            setattr(self.params, value_name, float(x))
            setattr(self.params, field_name, None)
        else:
            self._keep.append(x)
            setattr(self.params, field_name, x.data_ptr())

    def flux(self, grid, T, S, DIC=None, Alk=None, O2=None, out=None, stream=0):
        """Flux of every column (Ny, Nx) in FP64 from the surface cells of the 3-D fields."""
        import torch
        dt = A.F32 if T.dtype == torch.float32 else A.F64
        if out is None:
            out = torch.empty((grid.Ny, grid.Nx), dtype=torch.float64, device=T.device)
        ptr = lambda x: None if x is None else x.data_ptr()   # noqa: E731
        A.check(A.load().obgc_gas_exchange_flux(C.byref(self.params), C.byref(grid.c_grid()), dt, ptr(T), ptr(S),
                                                ptr(DIC), ptr(Alk), ptr(O2), out.data_ptr(), C.c_void_p(stream)),
                "obgc_gas_exchange_flux")
        return out

    def __call__(self, T, S, DIC=0.0, Alk=0.0, O2=0.0, u10=None, air=None):
        """One column on the host: the GasExchange functor's value."""
        f = C.c_double()
        A.check(A.load().obgc_gas_exchange_point(C.byref(self.params), float(T), float(S), float(DIC), float(Alk),
                                                 float(O2), self.params.wind_speed if u10 is None else float(u10),
                                                 self.params.air_concentration if air is None else float(air),
                                                 C.byref(f)), "obgc_gas_exchange_point")
        return f.value


def CarbonDioxideGasExchangeBoundaryCondition(**kw):
    """GasExchange.jl:96-124: pCO2 of the surface DIC/Alk against 413 ppmv, Ho06 k660, Wanninkhof
    (2014) CO2 Schmidt number, K0 rho / 1000 solubility."""
    return GasExchange(A.GAS_CO2, **kw)


def OxygenGasExchangeBoundaryCondition(**kw):
    """GasExchange.jl:126-146: surface O2 against 9352.7 mmol/m3 times the Wanninkhof (1992)
    solubility, Ho06 k660, Wanninkhof (2014) O2 Schmidt number."""
    return GasExchange(A.GAS_O2, **kw)

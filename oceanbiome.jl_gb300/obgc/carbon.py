"""CarbonChemistry mirror (src/Models/CarbonChemistry/carbon_chemistry.jl:66-218).

carbon_chemistry(; DIC, T, S, Alk, pH, P, output, silicate, phosphate) evaluates one point on the
host (FP64, same code as the device kernel) when given numbers, and solves every cell on the GPU
in FP64 when given device tensors.
"""
import ctypes as C

from . import _abi as A

_OUTPUTS = {"fCO2": A.OUT_FCO2, "fCO₂": A.OUT_FCO2, "pCO2": A.OUT_PCO2, "pCO₂": A.OUT_PCO2,
            "pHf": A.OUT_PH_FREE, "pHᶠ": A.OUT_PH_FREE, "pHt": A.OUT_PH_TOTAL, "pHᵗ": A.OUT_PH_TOTAL,
            "pHs": A.OUT_PH_SWS, "pHˢ": A.OUT_PH_SWS, "H": A.OUT_H, "CO3": A.OUT_CARBONATE,
            "Omega": A.OUT_OMEGA}


class CarbonChemistry:
    """Carbon chemistry model.  `density`: None for the reference's default
    teos10_polynomial_approximation (the TEOS-10 polynomial of Roquet et al. 2015), "eos80" for
    UNESCO EOS-80, or a constant density (kg/m3)."""

    def __init__(self, density=None, max_iters=100, atol=1e-20, initial_pH_guess=8.0, calcite_solubility="calcite"):
        """calcite_solubility: "calcite" (KSP_calcite, the default) or "aragonite" (KSP_aragonite):
        the solubility product of the saturation state Omega."""
        lib = A.load()
        self.options = A.CarbonOptions()
        A.check(lib.obgc_carbon_default_options(C.byref(self.options)), "obgc_carbon_default_options")
        self.options.max_iters = max_iters
        self.options.atol = atol
        self.options.initial_pH_guess = initial_pH_guess
        if density == "eos80":
            self.options.density = A.DENSITY_EOS80
        elif density is not None:
            self.options.density, self.options.density_value = A.DENSITY_CONSTANT, float(density)
        if calcite_solubility not in ("calcite", "aragonite"):
            raise ValueError("calcite_solubility is 'calcite' or 'aragonite'")
        self.options.saturation_mineral = int(calcite_solubility == "aragonite")

    def __repr__(self):
        return "`CarbonChemistry` model which solves for pCO₂ and pH"

    def _opts(self, output, pH, P):
        o = A.CarbonOptions()
        C.pointer(o)[0] = self.options
        o.output = _OUTPUTS[output] if isinstance(output, str) else int(output)
        o.ph_given = int(pH is not None)
        o.has_pressure = int(P is not None)
        return o

    def __call__(self, DIC, T, S, Alk=0.0, pH=None, P=None, output="fCO2", silicate=0.0, phosphate=0.0,
                 H=None, warm_start=False, iters=None, stream=0):
        o = self._opts(output, pH, P)
        lib = A.load()
        if isinstance(DIC, (int, float)):
            out = C.c_double(0)
            A.check(lib.obgc_carbon_chemistry_point(C.byref(o), float(DIC), float(Alk), float(T), float(S),
                                                    float(silicate), float(phosphate), float(P or 0.0),
                                                    float(pH or 0.0), C.byref(out)), "obgc_carbon_chemistry_point")
            return out.value
        import torch
        dt = A.F32 if DIC.dtype == torch.float32 else A.F64
        n = DIC.numel()
        out = torch.empty(n, dtype=torch.float64, device=DIC.device)
        o.warm_start = int(bool(warm_start))

        def ptr(x):
            return None if x is None or isinstance(x, (int, float)) else x.data_ptr()

        A.check(lib.obgc_carbon_chemistry(C.byref(o), n, dt, DIC.data_ptr(), ptr(Alk), T.data_ptr(), S.data_ptr(),
                                          ptr(silicate), ptr(phosphate), ptr(P), ptr(pH),
                                          None if H is None else H.data_ptr(), out.data_ptr(),
                                          None if iters is None else iters.data_ptr(), C.c_void_p(stream)),
                "obgc_carbon_chemistry")
        return out.view(DIC.shape)

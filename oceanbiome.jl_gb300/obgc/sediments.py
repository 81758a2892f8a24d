"""Sediment models below the water column (src/Models/Sediments, src/Sediments)."""


class InstantRemineralisationSediment:
    """InstantRemineralisationSediment(grid; sinking_tracers = (:P, :D), remineralisation_reciever
    = :N, burial_efficiency_constant1 = 0.013, burial_efficiency_constant2 = 0.53,
    burial_efficiency_half_saturation = 7.0 / 6.56) (instant_remineralisation.jl:56-120): the
    sinking flux F through the bottom face is buried with efficiency e = a + b (F / (k + F))^2 in a
    single-layer `storage` and the rest returns to the receiver in the bottom cell."""

    def __init__(self, grid=None, sinking_tracers=("P", "D"), remineralisation_reciever="N",
                 burial_efficiency_constant1=0.013, burial_efficiency_constant2=0.53,
                 burial_efficiency_half_saturation=7.0 / 6.56, timestepper="RungeKutta3"):
        self.grid = grid
        self.sinking_tracers = tuple(sinking_tracers)
        self.remineralisation_reciever = remineralisation_reciever
        self.a = float(burial_efficiency_constant1)
        self.b = float(burial_efficiency_constant2)
        self.k = float(burial_efficiency_half_saturation)
        self.timestepper = timestepper

    def summary(self):
        return "Single-layer instant remineralisation (Float64)"


class SimpleMultiGSediment:
    """SimpleMultiGSediment(grid; fast_decay_rate = 2/day, slow_decay_rate = 0.2/day, fast_fraction =
    0.74, slow_fraction = 0.26, refactory_fraction = 0.1, sedimentation_rate = 982 |z_bottom|^-1.548,
    anoxia_half_saturation = 1, sinking_nitrogen = (:sPOM, :bPOM), sinking_redfield = 6.56, the
    Soetaert et al. (2000) fit parameters) (src/Models/Sediments/simple_multi_G.jl:15-131), the
    nitrogen-only form: slow, fast and refractory sediment nitrogen fed by the sinking fluxes,
    remineralised into the bottom cell's NH4 and NO3 and drawing its O2.  Needs LOBSTER with Oxygen."""

    def __init__(self, grid=None, sinking_nitrogen=("sPOM", "bPOM"), sinking_carbon=None, **params):
        from . import _abi as A
        import ctypes as C
        if sinking_carbon is not None:
            raise NotImplementedError("the carbon form of SimpleMultiGSediment (sinking_carbon) in the fused step")
        self.grid = grid
        self.sinking_nitrogen = tuple(sinking_nitrogen)
        self.params = A.MultiGParams()
        A.check(A.load().obgc_multig_default_params(C.byref(self.params)), "obgc_multig_default_params")
        for k, v in params.items():
            if not hasattr(self.params, k):
                raise TypeError(f"unknown SimpleMultiGSediment parameter {k!r}")
            if isinstance(v, (tuple, list)):
                arr = getattr(self.params, k)
                for q in range(len(arr)):
                    arr[q] = float(v[q])
            else:
                setattr(self.params, k, float(v))

    def summary(self):
        return "Single-layer multi-G sediment model (Float64)"

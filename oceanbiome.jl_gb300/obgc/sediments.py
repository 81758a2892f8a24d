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

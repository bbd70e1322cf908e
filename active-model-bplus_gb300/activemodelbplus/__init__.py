"""GB300-native Active Model B+ (drop-in for the reference's ``activemodelbplus``
integrator package). The reference's mean-field theory modules (activedroplets,
activefield, ode, ...) are analytic side tools unrelated to the integrator and
are not part of this package."""

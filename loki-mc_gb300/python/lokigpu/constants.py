"""Physical constants and integer codes of the electron Monte Carlo path.

Values are those of the reference (Code/LoKI-MC/Headers/Constant.h:6-8, 23)
and its integer codes (Code/LoKI-MC/Headers/GeneralDefinitions.h:34-51);
they must match bit for bit.
"""

BOLTZMANN = 1.38064852e-23        # J/K
ELECTRON_CHARGE = 1.6021766208e-19  # C
ELECTRON_MASS = 9.10938356e-31     # kg
UNIFIED_ATOMIC_MASS = 1.660539040e-27  # kg
NON_DEF = -123456789.0

# process types
CONSERVATIVE = 0
IONIZATION = 1
ATTACHMENT = 2

# special process ids
NULL_COLLISION = -1
PARTIAL_FLIGHT = -2

# ionization energy sharing
EQUAL_SHARING = 0
ONE_TAKES_ALL = 1
USING_SDCS = 2
RANDOM_UNIFORM = 3

# gas temperature effect
GAS_TEMP_FALSE = 0
GAS_TEMP_TRUE = 1
GAS_TEMP_SMART = 2

# angular scattering samplers (Code/LoKI-MC/Headers/AngularScatteringFunctions.h:27-74)
SAMPLER_ISOTROPIC = 0
SAMPLER_FORWARD = 1
SAMPLER_BORN_DIPOLE = 2
SAMPLER_SURENDRA = 3
SAMPLER_COULOMB_SCREEN = 4
SAMPLER_MOMENTUM_CONSERVATION = 5

SAMPLER_NAMES = {
    "isotropic": SAMPLER_ISOTROPIC,
    "forward": SAMPLER_FORWARD,
    "bornDipole": SAMPLER_BORN_DIPOLE,
    "surendra": SAMPLER_SURENDRA,
    "coulombScreen": SAMPLER_COULOMB_SCREEN,
    "momentumConservationIonization": SAMPLER_MOMENTUM_CONSERVATION,
}

"""Physical constants and fit parameters used on the SIP hot path.

Units follow the reference model: particle masses in femtogram (1e-18 kg),
radii in micrometre, everything else SI.  Each value is the published physical
constant or material-fit coefficient the reference uses, and each derived value
is formed with the same floating-point operations as the reference so the bits
agree (reference files: constants.py, material_properties.py,
atmosphere.py:74-101,361-371, microphysics.py:970-1051,1355-1358,
integration.py:724-725).  ``csrc/lacmo_constants.h`` holds the same numbers as
hexadecimal literals for the CUDA kernels; ``tests/test_constants.py`` checks
that both agree.
"""
import math

import numpy as np

# constants.py
one_third = 1.0 / 3.0
four_pi_over_three = 4.0 * math.pi / 3.0
four_pi_over_three_inv = 0.75 / math.pi
earth_gravity = 9.80665
mass_density_water_liquid_NTP = 998.2
mass_density_air_dry_NTP = 1.2041
mass_density_NaCl_dry = 2163.0
mass_density_AS_dry = 1774.0
molar_mass_air_dry = 28.9644E-3
molar_mass_water = 18.015E-3
molar_mass_NaCl = 58.4428E-3
molar_mass_AS = 132.14E-3
universal_gas_constant = 8.3144598
specific_gas_constant_water_vapor = 461.53
specific_gas_constant_air_dry = 287.06
specific_heat_capacity_air_dry_NTP = 1004.71
specific_heat_capacity_water_vapor_20C = 1906
specific_heat_capacity_water_NTP = 4183.8

# atmosphere.py
kappa_air_dry = specific_gas_constant_air_dry / specific_heat_capacity_air_dry_NTP
epsilon_gc = specific_gas_constant_air_dry / specific_gas_constant_water_vapor
heat_factor_r_v = ((specific_heat_capacity_water_vapor_20C
                    - specific_gas_constant_water_vapor)
                   / (specific_heat_capacity_air_dry_NTP
                      - specific_gas_constant_air_dry))
kappa_factor = 1.0 / (1.0 - kappa_air_dry)
kappa_factor2 = -kappa_air_dry * kappa_factor

# material_properties.py
par_water_dens = np.array([1.00013502e+03, -4.68112708e-03, 2.72389977e+02])
par_sol_dens_NaCl = np.array([7.619443952135e+02, 1.021264281453e+03,
                              1.828970151543e+00, 2.405352122804e+02,
                              -1.080547892416e+00, -3.492805028749e-03])
par_rho_AS = np.array([997.1, 592., -5.036E1, 1.024E1])[::-1] / 997.1
par_sigma_NaCl = 1.62E-3 / molar_mass_NaCl / 0.072
par_sigma_AS = 2.362E-3 / molar_mass_AS / 0.072
w_s_max_NaCl = 0.45
w_s_max_AS = 0.78
par_wat_act_NaCl = np.array([1.0, -6.366E-1, 8.642E-1, -1.158E1, 1.518E1])[::-1]
par_wat_act_AS = np.array([1.0, -2.715E-1, 3.113E-1, -2.336, 1.412])[::-1]

# microphysics.py (Fukuta-Walter linearised size corrections, derivative fits)
accommodation_coeff = 1.0
adiabatic_index_inv = 0.7142857142857143
T_alpha_0 = 289.
c_alpha_1 = (1.0E6 * math.sqrt(2.0 * np.pi * specific_gas_constant_air_dry
                               * T_alpha_0)
             / (accommodation_coeff
                * (specific_heat_capacity_air_dry_NTP * adiabatic_index_inv
                   + 0.5 * specific_gas_constant_air_dry)))
c_alpha_2 = (0.5E6
             * math.sqrt(2.0 * np.pi * specific_gas_constant_air_dry / T_alpha_0)
             / (accommodation_coeff
                * (specific_heat_capacity_air_dry_NTP * adiabatic_index_inv
                   + 0.5 * specific_gas_constant_air_dry)))
condensation_coeff = 0.0415
c_beta_1 = (1.0E6 * math.sqrt(2.0 * np.pi * molar_mass_water
                              / (universal_gas_constant * T_alpha_0))
            / condensation_coeff)
c_beta_2 = -0.5 / T_alpha_0
par_rho_deriv_AS = np.copy(par_rho_AS[:-1]) * np.arange(1, len(par_rho_AS))[::-1]
par_wat_act_deriv_AS = (np.copy(par_wat_act_AS[:-1])
                        * np.arange(1, len(par_wat_act_AS))[::-1])
par_wat_act_deriv_NaCl = (np.copy(par_wat_act_NaCl[:-1])
                          * np.arange(1, len(par_wat_act_NaCl))[::-1])

# integration.py
w_s_max_NaCl_inv = 1. / w_s_max_NaCl
w_s_max_AS_inv = 1. / w_s_max_AS

SOLUTE_AS = 0
SOLUTE_NACL = 1


def solute_code(solute_type):
    """Map the reference's solute string ('AS' / 'NaCl') to the ABI code."""
    if solute_type == "AS":
        return SOLUTE_AS
    if solute_type == "NaCl":
        return SOLUTE_NACL
    raise ValueError(f"unknown solute_type {solute_type!r} (expected 'AS' or 'NaCl')")


def named_doubles():
    """All scalar constants shared with the CUDA header, by header name."""
    d = {
        "ONE_THIRD": one_third,
        "FOUR_PI_OVER_THREE": four_pi_over_three,
        "FOUR_PI_OVER_THREE_INV": four_pi_over_three_inv,
        "FOUR_PI": 4.0 * np.pi,
        "PI": math.pi,
        "R_V": specific_gas_constant_water_vapor,
        "R_D": specific_gas_constant_air_dry,
        "C_PD": specific_heat_capacity_air_dry_NTP,
        "KAPPA_AIR_DRY": kappa_air_dry,
        "EPSILON_GC": epsilon_gc,
        "HEAT_FACTOR_R_V": heat_factor_r_v,
        "KAPPA_FACTOR": kappa_factor,
        "KAPPA_FACTOR2": kappa_factor2,
        "PAR_SIGMA_AS": par_sigma_AS,
        "PAR_SIGMA_NACL": par_sigma_NaCl,
        "W_S_MAX_AS_INV": w_s_max_AS_inv,
        "C_ALPHA_1": c_alpha_1,
        "C_ALPHA_2": c_alpha_2,
        "C_BETA_1": c_beta_1,
        "C_BETA_2": c_beta_2,
        "T_ALPHA_0": T_alpha_0,
    }
    for k, v in enumerate(par_water_dens):
        d[f"PAR_WATER_DENS_{k}"] = float(v)
    for k, v in enumerate(par_sol_dens_NaCl):
        d[f"PAR_SOL_DENS_NACL_{k}"] = float(v)
    for k, v in enumerate(par_rho_AS):
        d[f"PAR_RHO_AS_{k}"] = float(v)
    for k, v in enumerate(par_rho_deriv_AS):
        d[f"PAR_RHO_DERIV_AS_{k}"] = float(v)
    for k, v in enumerate(par_wat_act_AS):
        d[f"PAR_WAT_ACT_AS_{k}"] = float(v)
    for k, v in enumerate(par_wat_act_deriv_AS):
        d[f"PAR_WAT_ACT_DERIV_AS_{k}"] = float(v)
    for k, v in enumerate(par_wat_act_NaCl):
        d[f"PAR_WAT_ACT_NACL_{k}"] = float(v)
    for k, v in enumerate(par_wat_act_deriv_NaCl):
        d[f"PAR_WAT_ACT_DERIV_NACL_{k}"] = float(v)
    return d

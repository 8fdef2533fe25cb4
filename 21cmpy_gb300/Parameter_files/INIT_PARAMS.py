"""Run parameters with the reference's names (Parameter_files/INIT_PARAMS.py:1-68).

The drop-in programs read these module globals exactly like the reference does; callers can
also pass overrides as keyword arguments.  Values are the reference's defaults except where the
reference's value is a machine path (IO_DIR defaults to the current directory).
"""
import numpy as np

IO_DIR = "."

DIM = np.int32(512)                # large (initial-conditions) box, pixels
HII_DIM = np.int32(128)
PIXEL_FACTOR = np.float32(DIM) / np.float32(HII_DIM)
MASS_FACTOR = np.float32(PIXEL_FACTOR ** 3.0)
BOX_LEN = np.float32(128)
DELTA_K = np.float32(2 * np.pi / BOX_LEN)
VOLUME = BOX_LEN * BOX_LEN * BOX_LEN
HII_TOT_NUM_PIXELS = HII_DIM * HII_DIM * HII_DIM
HII_shape = (HII_DIM, HII_DIM, HII_DIM)

INITIAL_REDSHIFT = 300.0
EVOLVE_DENSITY_LINEARLY = False
ION_Tvir_MIN = 1.0e4
ZETA = 40.0
R_BUBBLE_MAX = 30.0                # Mpc
R_BUBBLE_MIN = 0.5
FIND_BUBBLE_ALGORITHM = 0          # 0: centre pixel, 1: sphere painting
DELTA_R_FACTOR = 1.1

# 0 = real-space top-hat, 1 = k-space top-hat, 2 = Gaussian
HII_FILTER = 1
L_FACTOR = np.float32(0.620350491)

PLANCK13 = {"baryonic_effects": False, "omega_k_0": 0, "omega_M_0": 0.315, "omega_b_0": 0.0487,
            "n": 0.96, "N_nu": 0, "omega_lambda_0": 0.685, "omega_n_0": 0.0, "sigma_8": 0.829,
            "h": 0.673}
COSMO = PLANCK13

DIMENSIONAL_T_POWER_SPEC = False
T_USE_VELOCITIES = False
NUM_BINS = 100
USE_TS_IN_21CM = 0
ZETA_X = 2.0e56

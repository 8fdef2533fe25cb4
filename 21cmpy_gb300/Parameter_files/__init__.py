from .INIT_PARAMS import *  # noqa: F401,F403

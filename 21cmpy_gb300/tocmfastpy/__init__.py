from . import boxio  # noqa: F401

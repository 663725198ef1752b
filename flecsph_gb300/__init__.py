"""GB300-native SPH particle hot path (FleCSPH body-system / physics surface)."""
from . import abi  # noqa: F401

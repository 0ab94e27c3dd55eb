"""GB300-native drop-in for the EMT6-Ro Python package (python/emt6ro/__init__.py)."""
from . import simulation
from . import ga_model

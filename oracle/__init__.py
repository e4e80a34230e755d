"""CPU oracle of the spark timestep (test infrastructure; see oracle.py)."""
from .oracle import (Oracle, Mesh, Reference, RefIO, RefGrid, RNG_REFERENCE, RNG_PHILOX,  # noqa: F401
                     build)

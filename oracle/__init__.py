"""CPU oracle of the spark timestep (test infrastructure; see oracle.py)."""
from .oracle import Oracle, Mesh, Reference, RNG_REFERENCE, RNG_PHILOX, build  # noqa: F401

"""GB300-native SMAC + FENE-P + immersed-boundary time step (machapin/fortran8 hot path)."""
from . import abi
from .solver import CylSpec, F8Error, GridSpec, PhysSpec, Solver, State, empty_state

__all__ = ["abi", "CylSpec", "F8Error", "GridSpec", "PhysSpec", "Solver", "State", "empty_state"]

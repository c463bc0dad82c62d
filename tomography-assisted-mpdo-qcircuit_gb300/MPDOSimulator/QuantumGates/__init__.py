"""Quantum gates of the MPDO simulator (reference: MPDOSimulator/QuantumGates)."""
from .AbstractGate import QuantumGate, Truncate, Barrier  # noqa: F401

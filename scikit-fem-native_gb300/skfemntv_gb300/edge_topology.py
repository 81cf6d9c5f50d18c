"""Oriented edge topology (python/skfemntv/edge_topology.py), tetrahedra:
the module path the reference's callers import from."""
from .hcurl import OrientedEdgeTopology, build_oriented_edge_topology

__all__ = ["OrientedEdgeTopology", "build_oriented_edge_topology"]

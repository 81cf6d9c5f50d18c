"""Edge DOF map (python/skfemntv/edge_dof_map.py): the module path the
reference's callers import from."""
from .hcurl import OrientedEdgeDofMap, build_oriented_edge_dof_map

__all__ = ["OrientedEdgeDofMap", "build_oriented_edge_dof_map"]

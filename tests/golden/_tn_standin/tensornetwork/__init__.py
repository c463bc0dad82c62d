"""Stand-in for the part of the ``tensornetwork`` package that the reference
MPDO simulator calls (requirements.txt pins tensornetwork==0.4.6, which is not
installed in this environment).

Test infrastructure only: ``tests/golden/make_golden.py`` puts this directory
on ``sys.path`` so that the reference's own ``MPDOSimulator`` modules can run
and produce golden fixtures.  Nothing in the engine imports it.

What is restated here is the package's documented graph semantics, written
from scratch:

* ``Node(tensor, name, axis_names)`` owns one dangling ``Edge`` per axis, named
  by the axis name; ``node[name_or_index]`` returns the edge; ``axis_names`` is
  a plain list that callers may edit in place.
* ``connect`` / ``edge ^ edge`` joins two dangling edges; ``Edge.disconnect``
  splits a joined edge into two dangling ones that keep its name.
* ``contract(edge)`` and ``contract_between(a, b)`` contract the shared
  edge(s); the result's edges are ``a``'s remaining edges followed by ``b``'s,
  and the surviving ``Edge`` objects are re-pointed at the new node.
* ``contractors.*(nodes, output_edge_order=..., ignore_edge_order=...)``
  contract a whole network to one node.
* ``split_node`` transposes the node to (left edges, right edges), calls the
  backend ``svd(torch, tensor, pivot_axis, max_singular_values,
  max_truncation_error, relative)``, multiplies sqrt(s) into both factors and
  joins them by a new edge ``edge_name``; it returns (left, right,
  truncated singular values).  ``split_node_full_svd`` returns (U, S, V,
  truncated values) with S a diagonal node between edges ``left_edge_name``
  and ``right_edge_name``; ``split_node_qr`` calls the backend ``qr``.
* ``flatten_edges`` merges dangling edges of one node into one edge placed
  last, the first listed edge being the slowest-varying index.
* ``replicate_nodes`` copies nodes (sharing tensors) and the edges among them.

The backend arithmetic (``svd``/``qr``) is not restated: ``set_backend_module``
is handed the reference's own vendored ``decompositions.py``, which is the
file the package's pytorch backend would call.
"""
from typing import Any, List, Optional, Sequence

import torch

from . import contractors  # noqa: F401  (tn.contractors.auto / optimal)

_backend = None
_collections: List[Any] = []


def set_backend_module(mod) -> None:
    """Module providing ``svd(torch, ...)`` and ``qr(torch, ...)``."""
    global _backend
    _backend = mod


def set_default_backend(name) -> None:
    if name not in ('pytorch',):
        raise ValueError(f'only the pytorch backend is available, not {name!r}')


class Edge:
    def __init__(self, node1, axis1: int, name: Optional[str] = None, node2=None, axis2: Optional[int] = None):
        self.node1, self.axis1 = node1, axis1
        self.node2, self.axis2 = node2, axis2
        self.name = '__unnamed_edge__' if name is None else name

    def is_dangling(self) -> bool:
        return self.node2 is None

    def is_trace(self) -> bool:
        return self.node2 is self.node1

    @property
    def dimension(self) -> int:
        return int(self.node1.tensor.shape[self.axis1])

    def set_name(self, name: str) -> None:
        self.name = name

    def get_nodes(self):
        return [self.node1, self.node2]

    def __xor__(self, other: 'Edge') -> 'Edge':
        return connect(self, other)

    def disconnect(self, edge1_name: Optional[str] = None, edge2_name: Optional[str] = None):
        if self.is_dangling():
            raise ValueError('cannot disconnect a dangling edge')
        e1 = Edge(self.node1, self.axis1, name=edge1_name or self.name)
        e2 = Edge(self.node2, self.axis2, name=edge2_name or self.name)
        self.node1.edges[self.axis1] = e1
        self.node2.edges[self.axis2] = e2
        return e1, e2

    def _repoint(self, old_node, old_axis: int, new_node, new_axis: int) -> None:
        if self.node1 is old_node and self.axis1 == old_axis:
            self.node1, self.axis1 = new_node, new_axis
        elif self.node2 is old_node and self.axis2 == old_axis:
            self.node2, self.axis2 = new_node, new_axis
        else:
            raise ValueError('edge is not attached to that axis')

    def __repr__(self):
        return f'Edge({self.name!r})'


class AbstractNode:
    pass


class Node(AbstractNode):
    def __init__(self, tensor, name: Optional[str] = None, axis_names: Optional[Sequence[str]] = None,
                 backend: Any = None):
        if not torch.is_tensor(tensor):
            tensor = torch.as_tensor(tensor)
        self.tensor = tensor
        self.name = '__unnamed_node__' if name is None else name
        rank = tensor.dim()
        if axis_names is None:
            axis_names = [f'__unnamed_edge_{i}__' for i in range(rank)]
        if len(axis_names) != rank:
            raise ValueError(f'{len(axis_names)} axis names for a rank-{rank} tensor')
        self._axis_names = list(axis_names)
        self.edges: List[Edge] = [Edge(self, i, name=self._axis_names[i]) for i in range(rank)]
        for c in _collections:
            if isinstance(c, set):
                c.add(self)
            else:
                c.append(self)

    @property
    def axis_names(self) -> List[str]:
        return self._axis_names

    @axis_names.setter
    def axis_names(self, names):
        if len(names) != len(self.edges):
            raise ValueError('wrong number of axis names')
        self._axis_names = list(names)

    @property
    def shape(self):
        return tuple(self.tensor.shape)

    def get_rank(self) -> int:
        return self.tensor.dim()

    def set_tensor(self, tensor) -> None:
        self.tensor = tensor

    def set_name(self, name: str) -> None:
        self.name = name

    def get_axis_number(self, axis) -> int:
        if isinstance(axis, int):
            return axis
        return self._axis_names.index(axis)

    def __getitem__(self, key) -> Edge:
        if isinstance(key, int):
            return self.edges[key]
        try:
            return self.edges[self._axis_names.index(key)]
        except ValueError:
            raise ValueError(f'node {self.name!r} has no axis {key!r}; axes: {self._axis_names}') from None

    def _axis_of(self, edge: Edge) -> int:
        for i, e in enumerate(self.edges):
            if e is edge:
                return i
        raise ValueError(f'edge {edge.name!r} is not an edge of node {self.name!r}')

    def tensor_from_edge_order(self, edge_order: Sequence[Edge]):
        perm = [self._axis_of(e) for e in edge_order]
        if sorted(perm) != list(range(len(self.edges))):
            raise ValueError('edge order must list every edge of the node once')
        return self.tensor.permute(*perm)

    def reorder_edges(self, edge_order: Sequence[Edge]) -> 'Node':
        perm = [self._axis_of(e) for e in edge_order]
        self.tensor = self.tensor_from_edge_order(edge_order)
        old_edges = list(self.edges)
        # decide every endpoint before moving any (an edge's own axes are
        # compared against the old numbering)
        moves = []
        for new_axis, old_axis in enumerate(perm):
            e = old_edges[old_axis]
            first = e.node1 is self and e.axis1 == old_axis
            moves.append((e, first, new_axis))
        for e, first, new_axis in moves:
            if first:
                e.axis1 = new_axis
            else:
                e.axis2 = new_axis
        self._axis_names = [self._axis_names[p] for p in perm]
        self.edges = [old_edges[p] for p in perm]
        return self

    def copy(self, conjugate: bool = False) -> 'Node':
        t = self.tensor.conj() if conjugate else self.tensor
        n = Node(t, name=self.name, axis_names=list(self._axis_names))
        for i, e in enumerate(self.edges):
            n.edges[i].name = e.name
        return n

    def __repr__(self):
        return f'Node({self.name!r}, {self._axis_names}, {tuple(self.tensor.shape)})'


class NodeCollection:
    """Context manager: every Node created inside is added to ``container``."""

    def __init__(self, container):
        self.container = container

    def __enter__(self):
        _collections.append(self.container)
        return self

    def __exit__(self, *exc):
        _collections.remove(self.container)
        return False


def connect(edge1: Edge, edge2: Edge, name: Optional[str] = None) -> Edge:
    if edge1 is edge2:
        raise ValueError('cannot connect an edge to itself')
    if not edge1.is_dangling() or not edge2.is_dangling():
        raise ValueError('both edges must be dangling')
    if edge1.dimension != edge2.dimension:
        raise ValueError(f'dimension mismatch {edge1.dimension} != {edge2.dimension}')
    new = Edge(edge1.node1, edge1.axis1, name=name, node2=edge2.node1, axis2=edge2.axis1)
    edge1.node1.edges[edge1.axis1] = new
    edge2.node1.edges[edge2.axis1] = new
    return new


def _other_axis(edge: Edge, node) -> int:
    """Axis of ``edge`` on the endpoint that is not ``node`` (edge joins two nodes)."""
    return edge.axis2 if edge.node1 is node else edge.axis1


def _contract_pair(a: Node, b: Node, shared: Sequence[Edge], name: Optional[str]) -> Node:
    ax_a = [a._axis_of(e) for e in shared]
    ax_b = [_other_axis(e, a) for e in shared]
    t = torch.tensordot(a.tensor, b.tensor, dims=(ax_a, ax_b))
    keep_a = [i for i in range(len(a.edges)) if i not in ax_a]
    keep_b = [i for i in range(len(b.edges)) if i not in ax_b]
    ends = [(a, i) for i in keep_a] + [(b, i) for i in keep_b]
    new = Node(t, name=name, axis_names=[n.edges[i].name for n, i in ends])
    new.edges = [n.edges[i] for n, i in ends]
    for k, (n, i) in enumerate(ends):
        new.edges[k]._repoint(n, i, new, k)
    new._axis_names = [e.name for e in new.edges]
    return new


def contract(edge: Edge, name: Optional[str] = None, axis_names=None) -> Node:
    if edge.is_dangling():
        raise ValueError('cannot contract a dangling edge')
    if edge.is_trace():
        raise NotImplementedError('trace edges are not used by the reference path')
    return _contract_pair(edge.node1, edge.node2, [edge], name)


def contract_between(node1: Node, node2: Node, name: Optional[str] = None, allow_outer_product: bool = False,
                     output_edge_order=None, axis_names=None) -> Node:
    shared = [e for e in node1.edges if not e.is_dangling() and not e.is_trace()
              and (e.node1 is node2 or e.node2 is node2)]
    if not shared and not allow_outer_product:
        raise ValueError(f'no edges between {node1.name!r} and {node2.name!r}')
    out = _contract_pair(node1, node2, shared, name)
    if output_edge_order is not None:
        out.reorder_edges(output_edge_order)
    return out


def check_connected(nodes) -> None:
    nodes = list(nodes)
    if not nodes:
        return
    ids = {id(n) for n in nodes}
    seen = {id(nodes[0])}
    stack = [nodes[0]]
    while stack:
        n = stack.pop()
        for e in n.edges:
            if e.is_dangling():
                continue
            for m in (e.node1, e.node2):
                if id(m) in ids and id(m) not in seen:
                    seen.add(id(m))
                    stack.append(m)
    if len(seen) != len(ids):
        raise ValueError('Non-connected graph')


def replicate_nodes(nodes, conjugate: bool = False) -> List[Node]:
    nodes = list(nodes)
    copies = {id(n): n.copy(conjugate) for n in nodes}
    done = set()
    for n in nodes:
        for e in n.edges:
            if e.is_dangling() or id(e) in done:
                continue
            done.add(id(e))
            if id(e.node1) in copies and id(e.node2) in copies:
                c1, c2 = copies[id(e.node1)], copies[id(e.node2)]
                new = Edge(c1, e.axis1, name=e.name, node2=c2, axis2=e.axis2)
                c1.edges[e.axis1] = new
                c2.edges[e.axis2] = new
    return [copies[id(n)] for n in nodes]


def _split_inputs(node: Node, left_edges, right_edges):
    order = list(left_edges) + list(right_edges)
    t = node.tensor_from_edge_order(order)
    axes = [node._axis_of(e) for e in order]
    names = [node.axis_names[i] for i in axes]
    return t, axes, names[:len(left_edges)], names[len(left_edges):]


def _attach(new: Node, new_axis: int, edge: Edge, old: Node, old_axis: int) -> None:
    new.edges[new_axis] = edge
    edge._repoint(old, old_axis, new, new_axis)


def split_node(node: Node, left_edges, right_edges, max_singular_values: Optional[int] = None,
               max_truncation_err: Optional[float] = None, relative: bool = False, left_name: Optional[str] = None,
               right_name: Optional[str] = None, edge_name: Optional[str] = None):
    t, axes, lnames, rnames = _split_inputs(node, left_edges, right_edges)
    nl = len(left_edges)
    u, s, vh, trun = _backend.svd(torch, t, nl, max_singular_values, max_truncation_err, relative=relative)
    sq = torch.sqrt(s)
    u_s = u * sq
    vh_s = sq.reshape((-1,) + (1,) * (vh.dim() - 1)) * vh
    en = edge_name or '__unnamed_edge__'
    left = Node(u_s, name=left_name, axis_names=lnames + [en])
    right = Node(vh_s, name=right_name, axis_names=[en] + rnames)
    for i, e in enumerate(left_edges):
        _attach(left, i, e, node, axes[i])
    for i, e in enumerate(right_edges):
        _attach(right, i + 1, e, node, axes[nl + i])
    connect(left.edges[-1], right.edges[0], name=edge_name)
    node.edges = [Edge(node, i, name=nm) for i, nm in enumerate(node.axis_names)]
    return left, right, trun


def split_node_qr(node: Node, left_edges, right_edges, left_name: Optional[str] = None,
                  right_name: Optional[str] = None, edge_name: Optional[str] = None):
    t, axes, lnames, rnames = _split_inputs(node, left_edges, right_edges)
    nl = len(left_edges)
    q, r = _backend.qr(torch, t, nl)
    en = edge_name or '__unnamed_edge__'
    left = Node(q, name=left_name, axis_names=lnames + [en])
    right = Node(r, name=right_name, axis_names=[en] + rnames)
    for i, e in enumerate(left_edges):
        _attach(left, i, e, node, axes[i])
    for i, e in enumerate(right_edges):
        _attach(right, i + 1, e, node, axes[nl + i])
    connect(left.edges[-1], right.edges[0], name=edge_name)
    node.edges = [Edge(node, i, name=nm) for i, nm in enumerate(node.axis_names)]
    return left, right


def split_node_full_svd(node: Node, left_edges, right_edges, max_singular_values: Optional[int] = None,
                        max_truncation_err: Optional[float] = None, relative: bool = False,
                        left_name: Optional[str] = None, middle_name: Optional[str] = None,
                        right_name: Optional[str] = None, left_edge_name: Optional[str] = None,
                        right_edge_name: Optional[str] = None):
    t, axes, lnames, rnames = _split_inputs(node, left_edges, right_edges)
    nl = len(left_edges)
    u, s, vh, trun = _backend.svd(torch, t, nl, max_singular_values, max_truncation_err, relative=relative)
    ln = left_edge_name or '__unnamed_edge__'
    rn = right_edge_name or '__unnamed_edge__'
    left = Node(u, name=left_name, axis_names=lnames + [ln])
    mid = Node(torch.diag(s), name=middle_name, axis_names=[ln, rn])
    right = Node(vh, name=right_name, axis_names=[rn] + rnames)
    for i, e in enumerate(left_edges):
        _attach(left, i, e, node, axes[i])
    for i, e in enumerate(right_edges):
        _attach(right, i + 1, e, node, axes[nl + i])
    connect(left.edges[-1], mid.edges[0], name=left_edge_name)
    connect(mid.edges[1], right.edges[0], name=right_edge_name)
    node.edges = [Edge(node, i, name=nm) for i, nm in enumerate(node.axis_names)]
    return left, mid, right, trun


def flatten_edges(edges: Sequence[Edge], new_edge_name: Optional[str] = None) -> Edge:
    edges = list(edges)
    if not edges or any(not e.is_dangling() for e in edges):
        raise NotImplementedError('only dangling edges of one node are flattened on the reference path')
    node = edges[0].node1
    if any(e.node1 is not node for e in edges):
        raise ValueError('edges belong to different nodes')
    rest = [e for e in node.edges if all(e is not f for f in edges)]
    keep_names = [node.axis_names[node._axis_of(e)] for e in rest]
    node.reorder_edges(rest + edges)
    shape = tuple(node.tensor.shape)
    k = len(rest)
    node.tensor = node.tensor.reshape(shape[:k] + (-1,))
    new = Edge(node, k, name=new_edge_name)
    node.edges = rest + [new]
    node._axis_names = keep_names + [new.name]
    return new


__all__ = ['AbstractNode', 'Node', 'Edge', 'NodeCollection', 'connect', 'contract', 'contract_between',
           'contractors', 'check_connected', 'replicate_nodes', 'split_node', 'split_node_qr',
           'split_node_full_svd', 'flatten_edges', 'set_default_backend', 'set_backend_module']

"""Whole-network contraction (``tn.contractors.auto`` / ``optimal`` /
``greedy`` / ``branch``): every node of ``nodes`` is contracted into one node
whose edges are the subnetwork's open edges (dangling, or leading to a node
outside ``nodes``), in ``output_edge_order`` when given.  The path is left to torch.einsum (the result does not depend on it).
Test infrastructure for the golden-fixture generator only."""
from typing import Optional, Sequence


def _contract_all(nodes, output_edge_order: Optional[Sequence] = None, ignore_edge_order: bool = False,
                  memory_limit=None):
    import torch
    from . import Node
    nodes = list(nodes)
    ids = {id(n) for n in nodes}
    sym = {}
    dangling = []
    operands = []
    for n in nodes:
        sub = []
        for i, e in enumerate(n.edges):
            # open edges of the subnetwork: dangling ones and those that lead
            # to a node outside ``nodes`` (they stay attached to that node)
            if e.is_dangling() or id(e.node1) not in ids or id(e.node2) not in ids:
                dangling.append((e, n, i))
            if id(e) not in sym:
                sym[id(e)] = len(sym)
            sub.append(sym[id(e)])
        operands += [n.tensor, sub]
    if len(sym) > 52:
        raise ValueError('too many distinct edges for one einsum')
    if output_edge_order is not None:
        out_edges = list(output_edge_order)
        if {id(e) for e in out_edges} != {id(e) for e, _, _ in dangling}:
            raise ValueError('output_edge_order must list every dangling edge once')
    else:
        if len(dangling) > 1 and not ignore_edge_order:
            raise ValueError('the final node has more than one edge: give output_edge_order')
        out_edges = [e for e, _, _ in dangling]
    where = {id(e): (n, i) for e, n, i in dangling}
    t = torch.einsum(*operands, [sym[id(e)] for e in out_edges])
    new = Node(t, name='__contracted__', axis_names=[e.name for e in out_edges])
    new.edges = list(out_edges)
    for k, e in enumerate(out_edges):
        n, i = where[id(e)]
        e._repoint(n, i, new, k)
    return new


def auto(nodes, output_edge_order=None, memory_limit=None, ignore_edge_order: bool = False):
    return _contract_all(nodes, output_edge_order, ignore_edge_order)


def optimal(nodes, output_edge_order=None, memory_limit=None, ignore_edge_order: bool = False):
    return _contract_all(nodes, output_edge_order, ignore_edge_order)


def greedy(nodes, output_edge_order=None, memory_limit=None, ignore_edge_order: bool = False):
    return _contract_all(nodes, output_edge_order, ignore_edge_order)


def branch(nodes, output_edge_order=None, memory_limit=None, nbranch=None, ignore_edge_order: bool = False):
    return _contract_all(nodes, output_edge_order, ignore_edge_order)

"""Symbolic Hamiltonians and their TTNOs (``operators/hamiltonian.py``,
``ttno/ttno_class.py:60-97``).

A ``Hamiltonian`` is a sum of terms, each a tensor product of one-site
operators (matrices, or names looked up in ``conversion_dictionary``) times a
coefficient (a number, or a factor times a named coefficient from
``coeffs_mapping``). ``ttno_from_hamiltonian`` compiles it into a TTNO with a
finite-state construction of its own rather than the reference's state
diagrams: the state on the bond above node c is the part of a term that lies
in c's subtree (its "signature": which sites, which operators), with two
extra states, 0 = identity everywhere below and 1 = a complete term lies
below. Terms whose lower parts coincide share a state; a term's coefficient
is emitted at the lowest common ancestor of its sites. The TTNO is exact, so
any time evolution built on it gives the same result as on the reference's
TTNO for the same operator (the effective Hamiltonians are the same
operators); its bond dimensions can differ from the reference's minimal ones
when many terms overlap.
"""
from __future__ import annotations

from fractions import Fraction
from numbers import Number

import numpy as np

from .ttn import Node, TreeTensorNetworkOperator

ONE_SYMBOL = "1"


class Hamiltonian:
    """``Hamiltonian(terms, conversion_dictionary, coeffs_mapping)``: terms are
    TensorProducts (coefficient 1) or (factor, coefficient symbol, TensorProduct)."""

    def __init__(self, terms=None, conversion_dictionary: dict | None = None,
                 coeffs_mapping: dict | None = None):
        self.terms = _normalise_terms(terms)
        self.conversion_dictionary = {} if conversion_dictionary is None else dict(conversion_dictionary)
        self.coeffs_mapping = {} if coeffs_mapping is None else dict(coeffs_mapping)
        self.coeffs_mapping[ONE_SYMBOL] = 1

    def add_term(self, term):
        self.terms.extend(_normalise_terms(term))

    def add_multiple_terms(self, terms):
        self.terms.extend(_normalise_terms(list(terms)))

    def __add__(self, other: "Hamiltonian") -> "Hamiltonian":
        conv = dict(self.conversion_dictionary)
        conv.update(other.conversion_dictionary)
        coeffs = dict(self.coeffs_mapping)
        coeffs.update(other.coeffs_mapping)
        return Hamiltonian(list(self.terms) + list(other.terms), conv, coeffs)

    def __len__(self):
        return len(self.terms)

    def numeric_terms(self) -> list:
        """(complex coefficient, {node: matrix}) for every term."""
        out = []
        for factor, symbol, tp in self.terms:
            coeff = complex(factor) * complex(self.coeffs_mapping[symbol])
            ops = {}
            for nid, op in tp.items():
                if isinstance(op, str):
                    if op not in self.conversion_dictionary:
                        raise KeyError(f"operator {op!r} is not in the conversion dictionary")
                    op = self.conversion_dictionary[op]
                ops[nid] = np.asarray(op, dtype=complex)
            out.append((coeff, ops))
        return out


def _normalise_terms(terms) -> list:
    if terms is None:
        return []
    if isinstance(terms, dict):
        return [(Fraction(1), ONE_SYMBOL, terms)]
    if isinstance(terms, tuple) and len(terms) == 3 and not isinstance(terms[0], dict):
        return [terms]
    out = []
    for t in terms:
        if isinstance(t, dict):
            out.append((Fraction(1), ONE_SYMBOL, t))
        elif isinstance(t, tuple) and len(t) == 3 and isinstance(t[0], (Number, Fraction)):
            out.append(t)
        else:
            raise TypeError(f"a term must be a TensorProduct or (factor, symbol, TensorProduct), got {t!r}")
    return out


def _op_key(op: np.ndarray):
    a = np.ascontiguousarray(op, dtype=complex)
    return (a.shape, a.tobytes())


def ttno_from_hamiltonian(hamiltonian: Hamiltonian, reference_tree, dtype=complex) -> TreeTensorNetworkOperator:
    """The TTNO of ``hamiltonian`` on ``reference_tree``'s structure, legs
    (parent, children in the tree's physical order, out, in) per node."""
    tree = reference_tree
    tree._finalise()
    order = list(tree._order)
    parent = {n: tree.nodes[n].parent for n in order}
    kids = {n: list(tree.nodes[n].phys_children) for n in order}
    dim = {n: int(tree.phys(n).shape[-1]) for n in order}
    below = {}
    for n in reversed(_topological(order, parent, tree.root_id)):
        s = {n}
        for c in kids[n]:
            s |= below[c]
        below[n] = frozenset(s)
    depth = {tree.root_id: 0}
    for n in _topological(order, parent, tree.root_id):
        if parent[n] is not None:
            depth[n] = depth[parent[n]] + 1
    terms = []
    for coeff, ops in hamiltonian.numeric_terms():
        for nid, op in ops.items():
            if nid not in tree.nodes:
                raise ValueError(f"term acts on {nid}, which is not in the tree")
            if op.shape != (dim[nid], dim[nid]):
                raise ValueError(f"operator on {nid} has shape {op.shape}, expected {(dim[nid],) * 2}")
        terms.append((coeff, ops, frozenset(ops)))

    def lca(sites):
        if not sites:
            return tree.root_id
        paths = [tree.find_path_to_root(s) for s in sites]
        common = set(paths[0])
        for p in paths[1:]:
            common &= set(p)
        return max(common, key=lambda x: depth[x])

    def signature(ops, sites, c):
        return tuple(sorted((n, _op_key(ops[n])) for n in sites & below[c]))

    # bond states: signature -> index (2 + position), per child edge
    states = {c: {} for c in order if parent[c] is not None}
    for coeff, ops, sites in terms:
        for c in states:
            inter = sites & below[c]
            if inter and not sites <= below[c]:
                states[c].setdefault(signature(ops, sites, c), 2 + len(states[c]))
    ttno = TreeTensorNetworkOperator()
    for n in order:
        wp = None if parent[n] is None else 2 + len(states[n])
        wc = [2 + len(states[c]) for c in kids[n]]
        d = dim[n]
        eye = np.eye(d, dtype=complex)
        W = np.zeros(([wp] if wp is not None else []) + wc + [d, d], dtype=dtype)

        def put(bp, bc, op):
            W[tuple(([bp] if wp is not None else []) + list(bc) + [slice(None), slice(None)])] += op
        zero = [0] * len(kids[n])
        if wp is not None:
            put(0, zero, eye)
        for i in range(len(kids[n])):
            bc = list(zero)
            bc[i] = 1
            put(1, bc, eye)
        seen = set()
        for coeff, ops, sites in terms:
            top = lca(sites) == n
            crossing = wp is not None and bool(sites & below[n]) and not sites <= below[n]
            if not (top or crossing):
                continue
            child_states = [states[c][signature(ops, sites, c)] if sites & below[c] else 0 for c in kids[n]]
            local = ops.get(n, eye)
            if top:
                put(1, child_states, coeff * local)
            else:
                s = states[n][signature(ops, sites, n)]
                if s not in seen:          # one transition per shared lower part
                    seen.add(s)
                    put(s, child_states, local)
        node = Node(n)
        node.parent = parent[n]
        node.children = list(kids[n])
        node.phys_children = list(kids[n])
        node.shape = W.shape
        ttno.nodes[n] = node
        ttno._order.append(n)
        ttno._phys[n] = W
    ttno.root_id = tree.root_id
    return ttno


def _topological(order, parent, root):
    out, frontier = [root], [root]
    children = {n: [] for n in order}
    for n in order:
        if parent[n] is not None:
            children[parent[n]].append(n)
    while frontier:
        nxt = []
        for n in frontier:
            nxt += children[n]
        out += nxt
        frontier = nxt
    return out

"""Tree tensor network containers: TreeTensorNetworkState and TreeTensorNetworkOperator.

These mirror the construction API of PyTreeNet's ``TreeTensorNetwork``
(``core/ttn.py:117-1840``): ``add_root``, ``add_child_to_parent``, ``nodes``,
``tensors``, ``root_id``, ``orthogonality_center_id``. Storage differs: every
node tensor is kept in ONE physical leg layout -- (parent, children in the
order they were attached, open legs) -- on the GPU once an engine uses it. The
reference reorders a node's children as QR splits and contractions go by
(``core/ttn.py:1235-1313``, ``contractions/node_contraction.py:88-138``); that
*logical* order is tracked here as metadata (``Node.children``) because the
row order of each QR depends on it, and ``tensors[node_id]`` returns the
tensor permuted to the logical order, as the reference's lazy ``TensorDict``
(``core/ttn.py:72-115``) does.
"""
from __future__ import annotations

from collections.abc import Mapping
from typing import Iterator

import numpy as np


class Node:
    """A node of a tree: identifier, parent and (logical) children."""

    def __init__(self, identifier: str = "", tensor=None):
        self.identifier = str(identifier)
        self.parent: str | None = None
        self.children: list[str] = []          # logical (reference) order
        self.phys_children: list[str] = []     # physical layout order
        self.shape: tuple = tuple(np.shape(tensor)) if tensor is not None else ()

    def is_root(self) -> bool:
        return self.parent is None

    def is_leaf(self) -> bool:
        return len(self.children) == 0

    def nneighbours(self) -> int:
        return len(self.children) + (0 if self.parent is None else 1)

    def neighbouring_nodes(self) -> list[str]:
        """Logical order, parent first (``core/graph_node.py:340-355``)."""
        return ([self.parent] if self.parent is not None else []) + list(self.children)

    def phys_neighbours(self) -> list[str]:
        return ([self.parent] if self.parent is not None else []) + list(self.phys_children)

    def is_parent_of(self, other: str) -> bool:
        return other in self.children

    def is_child_of(self, other: str) -> bool:
        return self.parent == other

    def __repr__(self):
        return f"Node({self.identifier!r}, parent={self.parent!r}, children={self.children!r})"


class _TensorView(Mapping):
    """``ttn.tensors``: numpy arrays in the logical leg order of each node."""

    def __init__(self, ttn: "TreeTensorNetwork"):
        self._ttn = ttn

    def __getitem__(self, nid):
        return self._ttn.get_tensor(nid)

    def __setitem__(self, nid, value):
        self._ttn.set_tensor(nid, value)

    def __iter__(self) -> Iterator[str]:
        return iter(self._ttn._order)

    def __len__(self):
        return len(self._ttn._order)


class TreeTensorNetwork:
    """Common tree + tensor storage for states and operators."""

    n_open = 1

    def __init__(self):
        self.nodes: dict[str, Node] = {}
        self._order: list[str] = []
        self._phys: dict[str, object] = {}     # node id -> numpy or torch tensor, physical layout
        self.root_id: str | None = None
        self.orthogonality_center_id: str | None = None

    # -- construction (mirrors core/ttn.py:497-640) ---------------------------
    def add_root(self, node, tensor):
        node = node if isinstance(node, Node) else Node(node)
        if self.root_id is not None:
            raise ValueError("The tree already has a root")
        tensor = np.asarray(tensor)
        node.shape = tensor.shape
        node._open = list(range(tensor.ndim))   # leg indices of the given tensor still open
        node._legmap = []                       # physical leg -> index of the given tensor
        self.nodes[node.identifier] = node
        self._order.append(node.identifier)
        self._phys[node.identifier] = tensor
        self.root_id = node.identifier
        return node

    def add_child_to_parent(self, child, tensor, child_leg: int, parent_id: str, parent_leg: int,
                            compatible: bool = True):
        """Attach ``child`` below ``parent_id``. ``parent_leg`` indexes the parent's
        legs in the reference convention (parent, attached children, open legs)."""
        child = child if isinstance(child, Node) else Node(child)
        if child.identifier in self.nodes:
            raise ValueError(f"Node {child.identifier} already exists")
        parent = self.nodes[parent_id]
        tensor = np.asarray(tensor)
        nattached = (0 if parent.parent is None else 1) + len(parent.phys_children)
        open_idx = parent_leg - nattached
        if open_idx < 0 or open_idx >= len(parent._open) - self.n_open:
            raise ValueError(f"Leg {parent_leg} of {parent_id} is not an open virtual leg")
        if tensor.shape[child_leg] != parent.shape[parent._open[open_idx]]:
            raise ValueError("Bond dimensions of parent and child do not match")
        parent._legmap.append(parent._open.pop(open_idx))
        parent.phys_children.append(child.identifier)
        parent.children.append(child.identifier)
        child.parent = parent_id
        child.shape = tensor.shape
        child._open = [i for i in range(tensor.ndim) if i != child_leg]
        child._legmap = [child_leg]
        self.nodes[child.identifier] = child
        self._order.append(child.identifier)
        self._phys[child.identifier] = tensor
        return child

    def _finalise(self):
        """Permute every tensor given at construction into the physical layout."""
        for nid in self._order:
            node = self.nodes[nid]
            if hasattr(node, "_legmap"):
                perm = list(node._legmap) + list(node._open)
                t = self._phys[nid]
                self._phys[nid] = np.ascontiguousarray(np.transpose(t, perm))
                node.shape = self._phys[nid].shape
                del node._legmap, node._open

    # -- access ------------------------------------------------------------------
    @property
    def tensors(self) -> _TensorView:
        return _TensorView(self)

    def phys(self, nid):
        self._finalise()
        return self._phys[nid]

    def logical_perm(self, nid) -> list[int]:
        node = self.nodes[nid]
        off = 0 if node.parent is None else 1
        perm = list(range(off)) + [off + node.phys_children.index(c) for c in node.children]
        nv = off + len(node.children)
        return perm + list(range(nv, nv + self.n_open))

    def get_tensor(self, nid):
        t = self.phys(nid)
        if not isinstance(t, np.ndarray):
            t = t.detach().cpu().numpy()
        return np.transpose(t, self.logical_perm(nid))

    def set_tensor(self, nid, value):
        """Set a tensor given in the node's logical leg order. A node whose
        tensor lives on the device (the state of a running driver) is
        overwritten in place when the shape matches, so the engine's buffers
        keep their addresses (the drivers mutate their state in place, as in
        the reference)."""
        self._finalise()
        inv = [int(i) for i in np.argsort(self.logical_perm(nid))]
        cur = self._phys.get(nid)
        if cur is not None and not isinstance(cur, np.ndarray) and getattr(cur, "is_cuda", False):
            import torch
            src = value.permute(*inv) if isinstance(value, torch.Tensor) else \
                torch.from_numpy(np.ascontiguousarray(np.transpose(np.asarray(value), inv)))
            if tuple(src.shape) == tuple(cur.shape):
                cur.copy_(src)
                return
        self._phys[nid] = np.ascontiguousarray(np.transpose(np.asarray(value), inv))

    def __getitem__(self, nid):
        return self.nodes[nid], self.tensors[nid]

    def __contains__(self, nid):
        return nid in self.nodes

    # -- structure helpers (core/tree_structure.py) ----------------------------
    def phys_axis(self, nid, nbr) -> int:
        return self.nodes[nid].phys_neighbours().index(nbr)

    def find_path_to_root(self, nid) -> list[str]:
        path = [nid]
        while self.nodes[nid].parent is not None:
            nid = self.nodes[nid].parent
            path.append(nid)
        return path

    def path_from_to(self, a, b) -> list[str]:
        if a == b:
            return [a]
        pa, pb = self.find_path_to_root(a), self.find_path_to_root(b)
        sb = set(pb)
        lca = next(x for x in pa if x in sb)
        return pa[:pa.index(lca) + 1] + list(reversed(pb[:pb.index(lca)]))

    def distance_to_node(self, center) -> dict[str, int]:
        """Pre-order DFS over logical neighbours (``core/tree_structure.py:225-271``)."""
        out = {center: 0}

        def rec(nid, last, d):
            out[nid] = d
            for nb in self.nodes[nid].neighbouring_nodes():
                if nb != last:
                    rec(nb, nid, d + 1)
        for nb in self.nodes[center].neighbouring_nodes():
            rec(nb, center, 1)
        return out

    def get_leaves(self, include_root: bool = True) -> list[str]:
        """Leaf identifiers; with ``include_root`` a root with one neighbour
        counts too (``core/tree_structure.py:201-216``)."""
        leaves = [nid for nid in self._order if self.nodes[nid].is_leaf()]
        if include_root and self.root_id is not None and self.nodes[self.root_id].nneighbours() == 1:
            leaves.append(self.root_id)
        return leaves

    def get_leafs(self, include_root: bool = True) -> list[str]:
        return self.get_leaves(include_root=include_root)

    def is_child_of(self, pot_child: str, pot_parent: str) -> bool:
        """(``core/tree_structure.py:501-515``)"""
        return self.nodes[pot_child].parent == pot_parent

    def is_parent_of(self, pot_parent: str, pot_child: str) -> bool:
        return self.is_child_of(pot_child, pot_parent)

    def same_connectivity_as(self, other) -> bool:
        """Same node ids, same neighbours (``core/tree_structure.py:389-408``)."""
        if set(self.nodes) != set(other.nodes):
            return False
        return all(set(self.nodes[n].neighbouring_nodes()) == set(other.nodes[n].neighbouring_nodes())
                   for n in self.nodes)

    def same_hierarchy_as(self, other) -> bool:
        """Same parents and children (``core/tree_structure.py:410-431``)."""
        if set(self.nodes) != set(other.nodes):
            return False
        return all(self.nodes[n].parent == other.nodes[n].parent
                   and set(self.nodes[n].children) == set(other.nodes[n].children) for n in self.nodes)

    def _open_dims(self, nid) -> tuple:
        shape = self.phys(nid).shape
        return tuple(int(d) for d in shape[len(shape) - self.n_open:])

    def same_open_dimensions_as(self, other) -> bool:
        """Same open-leg dimensions on every node (``core/ttn.py:381-400``)."""
        if set(self.nodes) != set(other.nodes):
            return False
        return all(self._open_dims(n) == other._open_dims(n) for n in self.nodes)

    def same_structure_as(self, other) -> bool:
        """Same hierarchy and open dimensions (``core/ttn.py:338-356``)."""
        return self.same_hierarchy_as(other) and self.same_open_dimensions_as(other)

    def same_bond_dimensions_as(self, other) -> bool:
        """Same bond dimension on every edge (``core/ttn.py:358-379``)."""
        if not self.same_connectivity_as(other):
            return False
        return all(self.bond_dim(n, x) == other.bond_dim(n, x)
                   for n in self.nodes for x in self.nodes[n].neighbouring_nodes())

    def find_subtree_of_node(self, node_id: str) -> dict:
        """node id -> node for ``node_id`` and everything below it
        (``core/tree_structure.py:433-457``)."""
        out = {}

        def rec(n):
            out[n] = self.nodes[n]
            for c in self.nodes[n].children:
                rec(c)
        rec(node_id)
        return out

    def find_subtree_size_of_node(self, node_id: str) -> int:
        return len(self.find_subtree_of_node(node_id))

    def leaves_under_node(self, node_id: str) -> dict:
        """The leaves of ``node_id``'s subtree (``core/tree_structure.py:459-477``)."""
        return {n: node for n, node in self.find_subtree_of_node(node_id).items() if node.is_leaf()}

    def find_pairs_of_distance(self, distance: int, consider_open: bool = False) -> set:
        """Unordered pairs of nodes ``distance`` edges apart
        (``core/tree_structure.py:273-309``); with ``consider_open`` only nodes
        with an open leg of dimension above one count, and the distance is
        measured over those nodes alone."""
        def counts(n):
            return (not consider_open) or int(self.phys(n).shape[-1]) > 1
        if distance < 0:
            raise ValueError("distance must be non-negative")
        if distance == 0:
            return {frozenset([n]) for n in self._order if counts(n)}
        pairs = set()
        for a in self._order:
            if not counts(a):
                continue
            for b, d in self.distance_to_node(a).items():
                if b == a or not counts(b):
                    continue
                if consider_open:
                    path = self.path_from_to(a, b)
                    d = sum(1 for x in path[1:] if counts(x))
                if d == distance:
                    pairs.add(frozenset((a, b)))
        return pairs

    def nearest_neighbours(self, consider_open: bool = False) -> list:
        """Nearest-neighbour pairs (``core/tree_structure.py:187-199``)."""
        return [tuple(p) for p in self.find_pairs_of_distance(1, consider_open=consider_open)]

    def bond_dim(self, a, b) -> int:
        return self.phys(a).shape[self.phys_axis(a, b)]

    def pad_bond_dimension(self, node1_id: str, node2_id: str, new_bond_dim: int):
        """Zero-pad the bond between two neighbours to ``new_bond_dim`` (the old
        entries first), as ``core/ttn.py:792-836`` does with its projectors."""
        old = self.bond_dim(node1_id, node2_id)
        if new_bond_dim <= old:
            return
        for a, b in ((node1_id, node2_id), (node2_id, node1_id)):
            t = self.phys(a)
            ax = self.phys_axis(a, b)
            shape = list(t.shape)
            shape[ax] = new_bond_dim
            idx = tuple(slice(0, old) if i == ax else slice(None) for i in range(len(shape)))
            if isinstance(t, np.ndarray):
                out = np.zeros(shape, dtype=t.dtype)
            else:
                import torch
                out = torch.zeros(shape, dtype=t.dtype, device=t.device)
            out[idx] = t
            self._phys[a] = out
            self.nodes[a].shape = tuple(shape)

    def pad_bond_dimensions(self, new_bond_dim: int):
        """Every bond smaller than ``new_bond_dim`` padded to it (``core/ttn.py:838-863``)."""
        self._finalise()
        for n in self._order:
            p = self.nodes[n].parent
            if p is not None and self.bond_dim(n, p) < new_bond_dim:
                self.pad_bond_dimension(p, n, new_bond_dim)

    @property
    def root(self):
        """(root node, root tensor in its leg order) (``core/ttn.py:165-180``)."""
        if self.root_id is None:
            raise KeyError("There is no root in the TTN.")
        return self.nodes[self.root_id], self.get_tensor(self.root_id)

    def num_nodes(self) -> int:
        return len(self._order)

    def linearise(self, mode: str = "children_first") -> list:
        """Node order with every node after its children (or, with
        ``parents_first``, before them) (``core/tree_structure.py:653-690``)."""
        name = getattr(mode, "name", str(mode)).lower()
        out = []

        def rec(n):
            if name == "parents_first":
                out.append(n)
            for c in self.nodes[n].children:
                rec(c)
            if name != "parents_first":
                out.append(n)
        rec(self.root_id)
        return out

    def replace_tensor(self, node_id: str, new_tensor, permutation=None, new_shape: bool = False):
        """Set a node's tensor, given in its leg order (or permuted into it by
        ``permutation``) (``core/ttn.py:981-1010``)."""
        t = np.asarray(new_tensor) if not hasattr(new_tensor, "detach") else new_tensor.detach().cpu().numpy()
        if permutation is not None:
            t = np.transpose(t, permutation)
        if not new_shape and tuple(t.shape) != tuple(self.get_tensor(node_id).shape):
            raise ValueError("the new tensor does not fit the node (pass new_shape=True)")
        self.set_tensor(node_id, t)
        self.nodes[node_id].shape = tuple(self._phys[node_id].shape)

    def scale(self, factor, inplace: bool = True):
        """The network times ``factor``: the orthogonality centre's tensor (or
        the root's) is scaled, so a canonical form stays intact
        (``core/ttn.py:692-720``)."""
        ttn = self if inplace else self.copy_structure()
        if not inplace:
            ttn._phys = {k: (v.copy() if isinstance(v, np.ndarray) else v.clone()) for k, v in self._phys.items()}
        nid = ttn.orthogonality_center_id if ttn.orthogonality_center_id is not None else ttn.root_id
        if nid is None:
            raise AssertionError("Cannot scale an empty TTN!")
        ttn._phys[nid] = ttn._phys[nid] * factor
        return ttn

    def assert_orth_center(self, node_id: str, object_name: str = "tree tensor network"):
        """Raise unless ``node_id`` is the orthogonality centre (``core/ttn.py:1585-1600``)."""
        if self.orthogonality_center_id != node_id:
            raise AssertionError(f"The {object_name} has no orthogonality center at {node_id}!")

    def conjugate(self):
        """A copy with every tensor complex-conjugated (``core/ttn.py:681-690``)."""
        out = self.copy_structure()
        out._phys = {k: (np.conj(v) if isinstance(v, np.ndarray) else v.conj().resolve_conj())
                     for k, v in self._phys.items()}
        return out

    def _preorder(self) -> list:
        """Root first, then every child's subtree in the children's order."""
        self._finalise()
        out = []

        def rec(n):
            out.append(n)
            for c in self.nodes[n].children:
                rec(c)
        rec(self.root_id)
        return out

    def completely_contract_tree(self, to_copy: bool = False, order: list | None = None):
        """The whole network as one tensor and the node order of its open legs
        (``contractions/tree_contraction.py:20-62``): by default the nodes in
        the order the reference contracts them (root, then each child's subtree
        in turn); a state has one leg per node, an operator its (out, in) pair
        per node. Small trees only."""
        default = self._preorder()
        if order is None:
            order = default
        elif set(order) != set(default):
            raise ValueError("The order is inconsistent with the structure of the tree!")
        order = list(order)
        if hasattr(self, "to_dense"):
            vec = self.to_dense(order)
            dims = [int(self.phys(n).shape[-1]) for n in order]
            return vec.reshape(dims), order
        mat, _ = self.as_matrix(order)
        dims = [int(self.phys(n).shape[-2]) for n in order]
        n = len(order)
        pairs = [i for k in range(n) for i in (k, n + k)]
        return np.transpose(np.asarray(mat).reshape(dims + dims), pairs), order

    def bond_dims(self) -> dict:
        """(parent, child) -> bond dimension (``core/ttn.py:754-768``)."""
        return {(self.nodes[n].parent, n): self.bond_dim(n, self.nodes[n].parent)
                for n in self._order if self.nodes[n].parent is not None}

    def max_bond_dim(self) -> int:
        dims = self.bond_dims()
        if not dims:
            raise ValueError("This TTN has no virtual bond dimension!")
        return max(dims.values())

    def avg_bond_dim(self) -> float:
        dims = self.bond_dims()
        return sum(dims.values()) / len(dims)

    def size(self) -> int:
        return int(sum(int(np.prod(self.phys(n).shape)) for n in self._order))

    # -- files (``core/ttn.py:1747-1838``) ------------------------------------------
    def save(self, filepath: str):
        """``{filepath}.npz`` with every tensor in its node's leg order (parent,
        children in the node's order, open legs) and ``{filepath}.json`` with
        the structure (root, orthogonality centre, and per node identifier,
        parent, children, shape) -- PyTreeNet's format."""
        import json
        self._finalise()
        tensors = {nid: np.ascontiguousarray(self.get_tensor(nid)) for nid in self._order}
        np.savez(f"{filepath}.npz", **tensors)
        data = {"root_id": self.root_id,
                "orthogonality_center_id": self.orthogonality_center_id,
                "nodes": {nid: {"identifier": nid, "parent": self.nodes[nid].parent,
                                "children": list(self.nodes[nid].children),
                                "shape": list(tensors[nid].shape)} for nid in self._order}}
        with open(f"{filepath}.json", "w") as f:
            json.dump(data, f, indent=2)

    @classmethod
    def load(cls, filepath: str):
        """Read the two files written by :meth:`save` (or by PyTreeNet); every
        tensor is taken to be in its node's leg order."""
        import json
        import os
        if not (os.path.exists(f"{filepath}.npz") and os.path.exists(f"{filepath}.json")):
            raise FileNotFoundError(f"Could not find required files at {filepath}!")
        with open(f"{filepath}.json") as f:
            data = json.load(f)
        arrays = np.load(f"{filepath}.npz")
        ttn = cls()
        for nid, nd in data["nodes"].items():
            node = Node(nd["identifier"], arrays[nid])
            node.parent = nd["parent"]
            node.children = list(nd["children"])
            node.phys_children = list(nd["children"])
            ttn.nodes[nid] = node
            ttn._order.append(nid)
            ttn._phys[nid] = np.ascontiguousarray(arrays[nid])
        ttn.root_id = data["root_id"]
        ttn.orthogonality_center_id = data["orthogonality_center_id"]
        return ttn

    def copy_structure(self):
        """Deep copy of the structure (tensors are shared)."""
        import copy
        self._finalise()
        new = self.__class__.__new__(self.__class__)
        new.nodes = copy.deepcopy(self.nodes)
        new._order = list(self._order)
        new._phys = dict(self._phys)
        new.root_id = self.root_id
        new.orthogonality_center_id = self.orthogonality_center_id
        return new


class TreeTensorNetworkState(TreeTensorNetwork):
    """TTNS: one open (physical) leg per node (``ttns/ttns.py:18-444``)."""

    n_open = 1

    def to_complex(self, precision: int = 128) -> "TreeTensorNetworkState":
        """Stored tensors cast to complex128 (or complex64) (``ttns/ttns.py:423-444``);
        the engine computes in complex128 whatever the stored type."""
        if precision not in (64, 128):
            raise ValueError("Precision must be either 64 or 128!")
        dtype = np.complex128 if precision == 128 else np.complex64
        for nid, t in list(self._phys.items()):
            if hasattr(t, "detach"):
                import torch
                # device tensors stay where they are; only the dtype changes
                self._phys[nid] = t.to(torch.complex128 if precision == 128 else torch.complex64)
            else:
                self._phys[nid] = np.asarray(t).astype(dtype)
        return self

    def to_dense(self, site_order=None) -> np.ndarray:
        """Contract to a dense state vector (small trees only)."""
        self._finalise()
        site_order = site_order or list(self._order)

        def rec(nid, toward):
            A = np.asarray(self.get_phys_numpy(nid))
            legs = self.nodes[nid].phys_neighbours()
            cur = list(legs) + ["#" + nid]
            T = A
            for nb in legs:
                if nb == toward:
                    continue
                sub, subs = rec(nb, nid)
                ax = cur.index(nb)
                T = np.tensordot(T, sub, axes=([ax], [0]))
                cur = cur[:ax] + cur[ax + 1:] + ["#" + s for s in subs]
            if toward is not None:
                ax = cur.index(toward)
                T = np.moveaxis(T, ax, 0)
                cur = [cur[ax]] + cur[:ax] + cur[ax + 1:]
            return T, [c[1:] for c in cur if c.startswith("#")]
        T, sites = rec(self.root_id, None)
        return np.transpose(T, [sites.index(s) for s in site_order]).reshape(-1)

    # -- overlaps and expectation values on the engine (``ttns/ttns.py:49-297``) ------
    def _device(self):
        from .engine import DeviceNetwork
        return DeviceNetwork(self)

    def to_vector(self, to_copy: bool = False) -> tuple:
        """The dense state vector and the node order of its factors (small trees)."""
        return self.to_dense(list(self._order)), list(self._order)

    def scalar_product(self, other: "TreeTensorNetworkState | None" = None,
                       use_orthogonal_center: bool = True) -> complex:
        """sum self * conj(other) over all legs, i.e. <other|self>; <self|self>
        without ``other`` (``ttns.py:65-89``)."""
        mine = self._device()
        if other is None:
            return mine.expect_local({})
        return other._device().overlap(mine)

    def norm(self) -> float:
        return float(np.sqrt(self.scalar_product().real))

    def normalise(self, norm: float | None = None) -> float:
        """Divide the orthogonality centre (else the root) by the norm; returns the
        norm before (``ttns.py:91-125``)."""
        if norm is None:
            norm = self.norm()
        nid = self.orthogonality_center_id if self.orthogonality_center_id is not None else self.root_id
        if nid is None:
            raise ValueError("Cannot normalise TTNS without nodes!")
        self._phys[nid] = self.phys(nid) / norm
        return norm

    def normalize(self, norm: float | None = None) -> float:
        return self.normalise(norm)

    def distance(self, other: "TreeTensorNetworkState", normalise: bool = False) -> float:
        """||A - B|| with <A|B> taken in absolute value (``ttns.py:140-166``)."""
        a = self.scalar_product().real
        b = other.scalar_product().real
        dist = a - 2 * abs(self.scalar_product(other)) + b
        if dist < 0:
            assert dist > -1e-8 * min(a, b), f"Distance is negative! {dist}"
            dist = abs(dist)
        if normalise:
            dist *= 2 / (a + b)
        return float(np.sqrt(dist))

    def infidelity(self, other: "TreeTensorNetworkState") -> float:
        return 1 - self.distance(other, normalise=True)

    def single_site_operator_expectation_value(self, node_id: str, operator, move_orth_center: bool = False) -> complex:
        return self.tensor_product_expectation_value({node_id: operator})

    def tensor_product_expectation_value(self, operator) -> complex:
        """<psi| prod_i O_i |psi> (``ttns.py:240-264``)."""
        if len(operator) == 0:
            return self.scalar_product()
        return self._device().expect_local(dict(operator))

    # -- canonical forms on the device (``core/ttn.py:1530-1700``) -------------------
    def _orthogonalise(self, target: str, mode, full: bool):
        from .svd_truncation import SplitMode, TreeOps, canonical_form, move_center
        from .application import _device_tensor
        from . import engine as E
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("pytreenet_gb300 needs a CUDA device (no CPU fallback)")
        name = "REDUCED" if mode is None else getattr(mode, "name", str(mode)).upper()
        if name == "FULL":
            raise NotImplementedError("SplitMode.FULL is not provided")
        mode = SplitMode[name]
        dev = torch.device(E.DEFAULT_DEVICE)
        ops = TreeOps(self)
        with torch.no_grad():
            A = {n: _device_tensor(self.phys(n), dev) for n in self._order}
            if full or self.orthogonality_center_id is None:
                canonical_form(ops, A, target, reduced=mode is SplitMode.REDUCED)
            else:
                move_center(ops, A, self.orthogonality_center_id, target, reduced=mode is SplitMode.REDUCED)
        for n, t in A.items():
            self._phys[n] = t
            self.nodes[n].shape = tuple(t.shape)
        self.orthogonality_center_id = target

    def canonical_form(self, orthogonality_center_id: str, mode=None):
        """``TreeTensorNetwork.canonical_form``: moves an existing centre, else
        brings the whole network into canonical form (QR splits, ``mode``
        SplitMode.REDUCED by default or KEEP)."""
        self._orthogonalise(orthogonality_center_id, mode, full=False)

    def orthogonalize(self, orthogonality_center_id: str, mode=None):
        """``TreeTensorNetwork.orthogonalize`` (``core/ttn.py:1699-1715``): a
        wrapper of ``canonical_form`` (moves an existing centre, else brings the
        whole network into canonical form)."""
        self.canonical_form(orthogonality_center_id, mode=mode)

    def orthogonalize_from_scratch(self, orthogonality_center_id: str, mode=None):
        """Canonical form by QR splits of every node, whatever the current centre."""
        self._orthogonalise(orthogonality_center_id, mode, full=True)

    def orthogonalize_root(self, mode=None):
        """Canonical form with the centre at the root (``core/ttn.py:1652-1664``)."""
        if self.root_id is None:
            raise ValueError("The TTN has no root node!")
        self.canonical_form(self.root_id, mode=mode)

    def transpose_all_tensors(self):
        """Tensors are always served in their nodes' leg order; nothing to do
        (``core/ttn.py:1741-1746``)."""

    def move_orthogonalization_center(self, new_center_id: str, mode=None):
        if self.orthogonality_center_id is None:
            raise AssertionError("The TTN is not in canonical form, so the orth. center cannot be moved!")
        self._orthogonalise(new_center_id, mode, full=False)

    def ensure_orth_center(self, node_id: str, mode=None) -> bool:
        was = self.orthogonality_center_id == node_id
        if not was:
            self.canonical_form(node_id, mode)
        return was

    def ensure_root_orth_center(self, mode=None) -> bool:
        return self.ensure_orth_center(self.root_id, mode)

    def is_in_canonical_form(self, node_id: str | None = None) -> bool:
        """<psi|psi> equals the squared norm of the centre tensor (``ttns.py:299-327``)."""
        node_id = self.orthogonality_center_id if node_id is None else node_id
        if node_id is None:
            return False
        t = self.phys(node_id)
        t = t.detach().cpu().numpy() if not isinstance(t, np.ndarray) else t
        return bool(np.allclose(self.scalar_product(), np.vdot(t, t)))

    def multi_single_site_expectation_value(self, operators, move_orth: bool = False) -> dict:
        """node -> [<psi|O|psi> for each one-site operator on that node]
        (``ttns/ttns_util.py:25-175``): a TensorProduct is split into its
        one-site factors, a list groups single-site TensorProducts by node, a
        dict maps node -> TensorProduct or list of them. One device network
        serves all the contractions."""
        from .tdvp import TensorProduct

        def single(op):
            if len(op) != 1:
                raise ValueError("every operator must act on exactly one site")
            return op
        if isinstance(operators, TensorProduct):
            prepared = {n: [TensorProduct({n: o})] for n, o in operators.items()}
        elif isinstance(operators, list):
            prepared = {}
            for op in operators:
                n = next(iter(single(op)))
                prepared.setdefault(n, []).append(op)
        elif isinstance(operators, dict):
            prepared = {n: ([single(o) for o in op] if isinstance(op, list) else [single(op)])
                        for n, op in operators.items()}
        else:
            raise TypeError("Invalid input type of operators!")
        net = self._device()
        flat = [op for ops in prepared.values() for op in ops]
        vals = iter(net.expect_many(flat))
        return {n: [complex(next(vals)) for _ in ops] for n, ops in prepared.items()}

    def ttno_expectation_value(self, operator) -> complex:
        return self._device().expect_ttno(operator)

    def operator_expectation_value(self, operator) -> complex:
        """A TensorProduct (any mapping node -> matrix) or a TTNO (``ttns.py:278-297``)."""
        if isinstance(operator, TreeTensorNetworkOperator):
            return self.ttno_expectation_value(operator)
        if isinstance(operator, Mapping):
            return self.tensor_product_expectation_value(operator)
        raise TypeError("Operator must be a TensorProduct or a TTNO!")

    def apply_operator(self, operator):
        """Absorb every one-site operator of a TensorProduct into its node
        (``ttns.py:329-337``), on the device."""
        from .application import apply_operator_in_place
        apply_operator_in_place(self, operator)

    def get_phys_numpy(self, nid):
        t = self.phys(nid)
        return t if isinstance(t, np.ndarray) else t.detach().cpu().numpy()


class TreeTensorNetworkOperator(TreeTensorNetwork):
    """TTNO: two open legs (out, in) per node (``ttno/ttno_class.py:35-363``)."""

    n_open = 2

    def as_matrix(self, order: list | None = None):
        """The operator as a dense matrix and the node order of its factors
        (``ttno/ttno_class.py:44-58``); the contractions run on the device, for
        small trees only."""
        import torch
        from .adjoint import _raw_contract
        from .application import _device_tensor
        from . import engine as E
        if not torch.cuda.is_available():
            raise RuntimeError("pytreenet_gb300 needs a CUDA device (no CPU fallback)")
        dev = torch.device(E.DEFAULT_DEVICE)
        self._finalise()

        def rec(nid):
            node = self.nodes[nid]
            T = _device_tensor(self.phys(nid), dev)
            has_p = node.parent is not None
            kids = list(node.phys_children)
            n = T.dim() - 2
            labels = (["p"] if has_p else []) + [f"c{k}" for k in range(len(kids))] + ["t", "s"]
            sites = [nid]
            outs, ins = ["t"], ["s"]
            for k, c in enumerate(kids):
                sub, subsites = rec(c)
                new_labels = [l for l in labels if l != f"c{k}"] + [f"O{k}", f"I{k}"]
                T = _raw_contract(T, labels, sub, [f"c{k}", f"O{k}", f"I{k}"], new_labels, [f"c{k}"])
                labels = new_labels
                sites += subsites
                outs.append(f"O{k}")
                ins.append(f"I{k}")
            final = (["p"] if has_p else []) + outs + ins
            T = _raw_contract(T, labels, torch.ones((), dtype=T.dtype, device=dev), [], final, [])
            dim = int(np.prod([int(self.phys(x).shape[-1]) for x in sites]))
            shape = ([T.shape[0]] if has_p else []) + [dim, dim]
            return T.reshape(shape), sites
        mat, sites = rec(self.root_id)
        mat = mat.cpu().numpy()
        if order is None:
            return mat, sites
        dims = [int(self.phys(x).shape[-1]) for x in sites]
        perm = [sites.index(x) for x in order]
        nsite = len(sites)
        full = mat.reshape(dims + dims).transpose(perm + [nsite + i for i in perm])
        D = int(np.prod(dims))
        return full.reshape(D, D), list(order)

    @classmethod
    def from_hamiltonian(cls, hamiltonian, reference_tree, method=None, dtype=complex):
        """``TTNO.from_hamiltonian`` (``ttno/ttno_class.py:60-97``): the TTNO of a
        symbolic ``Hamiltonian`` on ``reference_tree``'s structure. ``method``
        (the reference's state-diagram finder) is accepted and not used: the
        construction of ``hamiltonian.ttno_from_hamiltonian`` is exact."""
        from .hamiltonian import ttno_from_hamiltonian
        return ttno_from_hamiltonian(hamiltonian, reference_tree, dtype=dtype)

    @classmethod
    def from_tensor(cls, reference_tree, tensor, leg_dict: dict, mode=None):
        """``TTNO.from_tensor`` (``ttno/ttno_class.py:163-298``): the TTNO of a
        dense operator tensor (legs out_1..out_n, in_1..in_n; ``leg_dict``
        maps node -> out leg) by successive device QR (default) or SVD splits."""
        from .ttno_decomposition import Decomposition, ttno_from_tensor
        return ttno_from_tensor(reference_tree, tensor, leg_dict, Decomposition.QR if mode is None else mode)


TTNS = TreeTensorNetworkState
TTNO = TreeTensorNetworkOperator

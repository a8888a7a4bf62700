"""Time-dependent TTNOs (``ttno/time_dep_ttno.py``).

The TDVP drivers with ``config.time_dep`` call ``update_hamiltonian`` after
every step and its measurement, as ``TimeEvolution.run`` does
(``time_evolution/time_evolution.py:346-368``): the TTNO advances by one time
step (``update``), may modify the state (``modify_state``), and the engine
copies the new TTNO tensors into the device buffers in place. The
environments are not rebuilt there (the reference does not rebuild them
either), so the next step starts from environments of the previous
Hamiltonian until the sweep renews them.

Tensor slices given to the updatables index the tensors in the reference's
leg order (parent, children in the node's order, out, in); the classes here
read and write them through a view of the engine's physical layout.
"""
from __future__ import annotations

from copy import deepcopy
from typing import Callable, Iterable

import numpy as np

from .ttn import TreeTensorNetworkOperator


def _as_slices(indices) -> tuple:
    return tuple(slice(i, i + 1) if isinstance(i, (int, np.integer)) else i for i in indices)


class AbstractTimeDepTTNO(TreeTensorNetworkOperator):
    """A TTNO whose tensors change with time (``time_dep_ttno.py:19-76``)."""

    def __init__(self, ttno: TreeTensorNetworkOperator | None = None):
        super().__init__()
        if ttno is not None:
            self._copy_ttno_attributes(ttno)

    def _copy_ttno_attributes(self, ttno: TreeTensorNetworkOperator):
        ttno._finalise()
        self.nodes = ttno.nodes
        self._order = ttno._order
        self._phys = ttno._phys
        self.root_id = ttno.root_id
        self.orthogonality_center_id = ttno.orthogonality_center_id

    def logical_view(self, nid) -> np.ndarray:
        """Writable view of node ``nid``'s tensor in the reference's leg order."""
        self._finalise()
        t = self._phys[nid]
        if not isinstance(t, np.ndarray):
            raise TypeError("time-dependent TTNO tensors must be NumPy arrays")
        return np.transpose(t, self.logical_perm(nid))

    def update(self, time_step_size: float):
        raise NotImplementedError("This method must be implemented in a subclass!")

    def reset(self):
        raise NotImplementedError("This method must be implemented in a subclass!")

    def modify_state(self, state):
        raise NotImplementedError("This method must be implemented in a subclass!")


class FactorUpdatable:
    """Values f(t) * A on a slice of one node's tensor (``time_dep_ttno.py:370-470``)."""

    def __init__(self, node_id: str, indices: tuple, initial_values: np.ndarray,
                 factor_function: Callable[[float], complex]):
        self.node_id = node_id
        self._indices = _as_slices(indices)
        if len(self._indices) != np.ndim(initial_values):
            raise AssertionError("The number of indices must match the number of dimensions of the tensor!")
        self.initial_values = np.asarray(initial_values)
        self.factor_function = factor_function
        self.current_time = 0.0
        self.current_values = factor_function(0) * self.initial_values

    @property
    def indices(self) -> tuple:
        return self._indices

    @property
    def shape(self) -> tuple:
        return self.initial_values.shape

    def update_current_time(self, time_step_size: float):
        self.current_time += time_step_size

    def update(self, time_step_size: float):
        self.update_current_time(time_step_size)
        self.current_values = self.factor_function(self.current_time) * self.initial_values

    def get_zero_time_values(self):
        return self.factor_function(0) * self.initial_values


class TimeDependentTTNO(AbstractTimeDepTTNO):
    """TTNO tensors = values without the updatables + the updatables' current
    values (``TimeDependentTTNO``, ``time_dep_ttno.py:211-342``)."""

    def __init__(self, updatables: Iterable, ttno: TreeTensorNetworkOperator | None = None):
        super().__init__(ttno=ttno)
        updatables = tuple(updatables)
        self.updatable_check(updatables)
        self.updatables = updatables
        self.orig_values = tuple((deepcopy(self.logical_view(u.node_id)[u.indices]), u.node_id, u.indices)
                                 for u in updatables)
        self.fill_tensors()

    def updatable_check(self, updatables):
        for u in updatables:
            if u.node_id not in self.nodes:
                raise ValueError(f"Node id {u.node_id} not found in the TTNO.")
            shape = self.logical_view(u.node_id).shape
            if len(shape) != len(u.indices):
                raise ValueError(f"Shape of node {u.node_id} does not match the shape of the updatable.")
            for i, index in enumerate(u.indices[:-2]):
                start = 0 if index.start is None else index.start
                stop = shape[i] if index.stop is None else index.stop
                if stop > shape[i] or start < 0:
                    raise ValueError(f"Index {index} is out of bounds for node {u.node_id}.")

    def update(self, time_step_size: float):
        self.reset_tensors()
        for u in self.updatables:
            u.update(time_step_size)
        self.fill_tensors()

    def reset_tensors(self):
        for values, nid, idx in self.orig_values:
            self.logical_view(nid)[idx] = values

    def fill_tensors(self):
        for u in self.updatables:
            self.logical_view(u.node_id)[u.indices] += u.current_values

    def reset(self):
        self.reset_tensors()

    def modify_state(self, state):
        pass


class DiscreetTimeTTNO(AbstractTimeDepTTNO):
    """A TTNO that switches to the next of a list every ``dt`` of time
    (``DiscreetTimeTTNO``, ``time_dep_ttno.py:87-209``). Measurements between
    the switches are not provided: ``measurements`` must be None."""

    def __init__(self, ttnos: list, dt: float = 1.0, measurements=None):
        if measurements is not None:
            raise NotImplementedError("measurements between TTNO switches are not provided")
        super().__init__(ttno=ttnos[0])
        self.ttnos = ttnos
        self.current_time_step = 0
        self.current_time = 0
        self.dt = dt

    def set_ttno_to_time_step(self, time_step: int):
        if time_step < 0 or time_step >= len(self.ttnos):
            raise ValueError(f"Time step {time_step} is out of bounds.")
        self._copy_ttno_attributes(self.ttnos[time_step])

    def update(self, time_step_size: float):
        self.current_time += time_step_size
        if self.current_time_step < len(self.ttnos) - 1 and \
                self.current_time >= (self.current_time_step + 1) * self.dt:
            self.current_time_step += 1
            self.set_ttno_to_time_step(self.current_time_step)

    def reset(self):
        self.current_time_step = 0
        self.current_time = 0
        self.set_ttno_to_time_step(0)

    def modify_state(self, state):
        pass

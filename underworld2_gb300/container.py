"""Index sets (``uw.container``, P/container/_indexset.py:20-650).

A set of non-negative integers below ``size``, held as a boolean mask on the
host; members come back as a read-only uint32 array in increasing order, as
the reference's StGermain IndexSet returns them.  The operators follow the
reference: ``+``/``|`` union, ``-`` difference, ``&`` intersection (and their
in-place forms), ``invert``, ``addAll``, ``clear``, ``AND``; operands must be
of the same type and size.
"""
import copy
import numbers

import numpy as np


class IndexSet:
    """The IndexSet container (P/container/_indexset.py:20-604)."""

    _size = 0
    _mask = np.zeros(0, dtype=bool)
    _data = None

    def __init__(self, size, fromObject=None):
        if not isinstance(size, numbers.Integral) or isinstance(size, bool):
            raise ValueError("The 'size' parameter must be of type int.")
        if size <= 0:
            raise ValueError("The 'size' parameter must be positive.")
        self._size = int(size)
        self._mask = np.zeros(self._size, dtype=bool)
        self._data = None
        if fromObject is not None:
            self.add(fromObject)

    @property
    def size(self):
        """The largest index the set can hold, plus one (not the member count)."""
        return self._size

    def _as_indices(self, indices):
        if isinstance(indices, numbers.Integral) and not isinstance(indices, bool):
            i = int(indices)
            if i >= self._size or i < 0:
                raise ValueError("Provided index must be non-negative and less than IndexSet maximum ({})."
                                 .format(self._size - 1))
            return np.array([i], dtype=np.int64)
        if isinstance(indices, IndexSet):
            self._checkCompatWith(indices)
            return np.flatnonzero(indices._mask)
        if not isinstance(indices, np.ndarray):
            try:
                indices = np.fromiter(iter(indices), dtype=np.int64)
            except TypeError:
                raise TypeError("The object passed in does not appear to be iterable or other compatible type.")
        if indices.size == 0:
            return np.zeros(0, dtype=np.int64)
        if not np.issubdtype(indices.dtype, np.integer):
            raise TypeError("Incompatible array type ({}) provided. Must be of integer type.".format(indices.dtype))
        if indices.max() > self._size - 1:
            raise ValueError("Provided object contains a value ({}) greater than the IndexSet maximum ({})."
                             .format(indices.max(), self._size - 1))
        if indices.min() < 0:
            raise ValueError("Provided object contains a value ({}) less than zero.".format(indices.min()))
        return indices.astype(np.int64).ravel()

    def add(self, indices):
        """Add an index, an iterable or array of indices, or another set's members."""
        self._mask[self._as_indices(indices)] = True
        self._data = None

    def remove(self, indices):
        """Remove an index, an iterable or array of indices, or another set's members."""
        self._mask[self._as_indices(indices)] = False
        self._data = None

    def AND(self, indices):
        """Keep only the members also in the IndexSet `indices`."""
        self._checkCompatWith(indices)
        self._mask &= indices._mask
        self._data = None

    def __contains__(self, index):
        i = int(index)
        return 0 <= i < self._size and bool(self._mask[i])

    def __getitem__(self, index):
        return self.data[index]

    @property
    def data(self):
        """Members as a read-only uint32 array."""
        if self._data is None:
            arr = np.flatnonzero(self._mask).astype(np.uint32)
            arr.flags.writeable = False
            self._data = arr
        return self._data

    def __len__(self):
        return int(np.count_nonzero(self._mask))

    def invert(self):
        self._mask = ~self._mask
        self._data = None

    def addAll(self):
        self._mask[:] = True
        self._data = None

    def clear(self):
        self._mask[:] = False
        self._data = None

    def __repr__(self):
        return repr(self.data).replace("array", type(self).__name__).replace(", dtype=uint32", "")

    def __iter__(self):
        return iter(self.data)

    def _binary(self, other, op):
        if not isinstance(other, IndexSet):
            raise TypeError("Indices provided must be of type 'IndexSet'.")
        self._checkCompatWith(other)
        out = copy.deepcopy(self)
        out._mask = op(out._mask, other._mask)
        out._data = None
        return out

    def __add__(self, other):
        return self._binary(other, np.logical_or)

    def __or__(self, other):
        return self._binary(other, np.logical_or)

    def __sub__(self, other):
        return self._binary(other, lambda a, b: a & ~b)

    def __and__(self, other):
        return self._binary(other, np.logical_and)

    def __iadd__(self, other):
        r = self._binary(other, np.logical_or)
        self._mask, self._data = r._mask, None
        return self

    __ior__ = __iadd__

    def __isub__(self, other):
        r = self._binary(other, lambda a, b: a & ~b)
        self._mask, self._data = r._mask, None
        return self

    def __iand__(self, other):
        r = self._binary(other, np.logical_and)
        self._mask, self._data = r._mask, None
        return self

    def __deepcopy__(self, memo):
        new = copy.copy(self)
        new._mask = self._mask.copy()
        new._data = None
        return new

    def _checkCompatWith(self, other):
        if type(self) != type(other):
            raise TypeError("This operation is illegal. These objects do not appear to be of identical type.")
        if self._size != other._size:
            raise ValueError("This operation is illegal. These IndexSets have different sizes.")


class ObjectifiedIndexSet(IndexSet):
    """An IndexSet tied to the object its indices refer to (P/container/_indexset.py:605-650)."""

    def __init__(self, object=None, *args, **kwargs):
        self._object = object
        super().__init__(*args, **kwargs)

    @property
    def object(self):
        return self._object

    def _checkCompatWith(self, other):
        super()._checkCompatWith(other)
        if self._object is not other._object:
            raise TypeError("This operation is illegal. These objects do not appear to be related to the same "
                            "object.")

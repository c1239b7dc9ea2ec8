"""Plan caches keyed on tensor identity.

Solver plans (children CSR of a tree, the target CSR of a connection list,
tap plans of a delay ring) are derived from small index tensors and reused
across calls.  A key made of ``data_ptr()`` and ``_version`` is unsafe: once
a tensor is freed, the caching allocator hands its address to the next
tensor of the same size, whose version starts at 0 again, so a lookup would
return the plan of a different topology.  Entries here hold the key tensors
themselves and match them by identity (and version), so an address cannot be
reused while its entry exists.
"""

from __future__ import annotations

from collections import OrderedDict


class TensorKeyedCache:
    """A small LRU map from (tensors by identity and version, extra key) to a value."""

    def __init__(self, capacity: int = 32):
        self.capacity = int(capacity)
        self._entries: OrderedDict = OrderedDict()
        self._serial = 0

    @staticmethod
    def _versions(tensors):
        return tuple(None if t is None else t._version for t in tensors)

    def get(self, tensors, extra, build):
        """The cached value for ``tensors`` (a tuple; entries may be None) and
        the hashable ``extra``, else ``build()`` stored under them."""
        tensors = tuple(tensors)
        vers = self._versions(tensors)
        for slot, (held, held_vers, held_extra, value) in self._entries.items():
            if (held_extra == extra and held_vers == vers and len(held) == len(tensors)
                    and all(a is b for a, b in zip(held, tensors))):
                self._entries.move_to_end(slot)
                return value
        value = build()
        self._serial += 1
        self._entries[self._serial] = (tensors, vers, extra, value)
        while len(self._entries) > self.capacity:
            self._entries.popitem(last=False)
        return value

    def clear(self):
        self._entries.clear()

    def __len__(self):
        return len(self._entries)

"""A stim-format detector error model returned when stim is not importable.

Mirrors what the reference returns (a ``stim.DetectorErrorModel`` with one
``error(p) D.. L..`` instruction per merged symptom, Driver.hpp:166-194):
``num_errors``, ``num_detectors``, ``num_observables``, text form, ``==``
(instruction order and exact probabilities, like stim) and ``approx_equals``.
"""

from __future__ import annotations

import numpy as np


class DetectorErrorModel:
    """Merged error mechanisms as CSR arrays (targets >= num_detectors are observables)."""

    def __init__(self, probs, offsets, targets, num_detectors: int, num_observables: int,
                 num_raw_mechanisms: int = 0):
        self._arrays = (np.asarray(probs, dtype=np.float64), np.asarray(offsets, dtype=np.uint32),
                        np.asarray(targets, dtype=np.uint32))
        self._loader = None
        self._num_detectors = int(num_detectors)
        self._num_observables = int(num_observables)
        self.num_raw_mechanisms = int(num_raw_mechanisms)

    @classmethod
    def _deferred(cls, loader, num_detectors: int, num_observables: int, num_raw_mechanisms: int):
        """A DEM whose arrays ``loader()`` returns as (probs, offsets, targets) views on first use
        (the data already sits in host memory; only the views are deferred)."""
        self = cls.__new__(cls)
        self._arrays = None
        self._loader = loader
        self._num_detectors = int(num_detectors)
        self._num_observables = int(num_observables)
        self.num_raw_mechanisms = int(num_raw_mechanisms)
        return self

    def _views(self):
        if self._arrays is None:
            self._arrays = self._loader()
            self._loader = None
        return self._arrays

    @property
    def probs(self) -> np.ndarray:
        return self._views()[0]

    @property
    def offsets(self) -> np.ndarray:
        return self._views()[1]

    @property
    def targets(self) -> np.ndarray:
        return self._views()[2]

    @property
    def num_errors(self) -> int:
        return int(self.probs.shape[0])

    @property
    def num_detectors(self) -> int:
        return self._num_detectors

    @property
    def num_observables(self) -> int:
        return self._num_observables

    def errors(self):
        """Yields (targets tuple, p) in instruction order."""
        off = self.offsets
        tg = self.targets
        for i in range(self.num_errors):
            yield tuple(int(t) for t in tg[off[i]:off[i + 1]]), float(self.probs[i])

    def named_errors(self):
        """Yields (('D3', 'D7', 'L0'), p) in instruction order."""
        nd = self._num_detectors
        for ts, p in self.errors():
            yield tuple([f"D{t}" for t in ts if t < nd] + [f"L{t - nd}" for t in ts if t >= nd]), p

    def canonical(self):
        """Order-free form: sorted list of (targets tuple, p)."""
        return sorted(self.errors())

    def __str__(self) -> str:
        lines = []
        for names, p in self.named_errors():
            lines.append(f"error({p!r}) " + " ".join(names))
        return "\n".join(lines) + ("\n" if lines else "")

    def __repr__(self) -> str:
        return f"DetectorErrorModel(num_errors={self.num_errors}, num_detectors={self.num_detectors})"

    def __eq__(self, other) -> bool:
        if not isinstance(other, DetectorErrorModel):
            return NotImplemented
        return (self._num_detectors == other._num_detectors
                and self._num_observables == other._num_observables
                and np.array_equal(self.offsets, other.offsets)
                and np.array_equal(self.targets, other.targets)
                and np.array_equal(self.probs, other.probs))

    def approx_equals(self, other, *, atol: float = 0.0, rtol: float = 1e-12, ordered: bool = False) -> bool:
        """Same symptom sets and probabilities within tolerance (order-free unless ``ordered``)."""
        a = list(self.errors()) if ordered else self.canonical()
        b = list(other.errors()) if ordered else other.canonical()
        if len(a) != len(b):
            return False
        for (ta, pa), (tb, pb) in zip(a, b):
            if ta != tb or abs(pa - pb) > atol + rtol * abs(pb):
                return False
        return True

    def to_stim(self):
        """The same model as a stim.DetectorErrorModel (requires stim)."""
        import stim
        return stim.DetectorErrorModel(str(self))

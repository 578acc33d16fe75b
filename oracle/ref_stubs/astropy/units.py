"""Minimal unit objects for loading the reference's Cython module.

fast_likelihood.pyx reads ``u.day``, ``u.one`` and ``u.radian`` at import time
(:42-45) and builds units with ``/`` and ``**`` in ``CJokerHelper.__init__``
(:139-148, :166).  Values handed to the helper are already in the internal
units, so a unit here is only a label.
"""


class Unit:
    def __init__(self, name):
        self.name = name

    def __truediv__(self, other):
        return Unit(f"({self.name})/({getattr(other, 'name', other)})")

    def __rtruediv__(self, other):
        return Unit(f"({other})/({self.name})")

    def __mul__(self, other):
        return Unit(f"({self.name})*({getattr(other, 'name', other)})")

    __rmul__ = __mul__

    def __pow__(self, p):
        return Unit(f"({self.name})**{p}")

    def __repr__(self):
        return f"Unit({self.name})"


day = Unit("d")
one = Unit("")
radian = Unit("rad")
km = Unit("km")
s = Unit("s")

"""Stand-in for thejoker.distributions; the Cython helper imports the name
FixedCompanionMass (fast_likelihood.pyx:224) but only inspects the K prior's
``owner.op._print_name`` (:225)."""


class FixedCompanionMass:
    pass

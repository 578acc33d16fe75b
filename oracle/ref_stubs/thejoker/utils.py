"""Stand-in for thejoker.utils._pytensor_get_mean_std.

The reference evaluates a pymc Normal's mean and standard deviation and converts
them between units (thejoker/utils.py).  The oracle's prior objects carry those
two numbers directly, already in the internal units."""


def _pytensor_get_mean_std(dist, in_unit, out_unit):
    return float(dist.mean), float(dist.std)

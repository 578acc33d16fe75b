"""Import-time stand-in for astropy, used only to load the reference's compiled
Cython likelihood in the oracle.  Only ``astropy.units`` is provided."""

"""Import-time stand-in for the reference package, so that its compiled
``thejoker.src.fast_likelihood`` extension can be loaded by the oracle."""

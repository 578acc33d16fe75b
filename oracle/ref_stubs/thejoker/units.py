"""Stand-in for thejoker.units: the attribute name under which a prior
variable carries its unit (the reference uses the same string)."""

UNIT_ATTR_NAME = "__tensor_unit__"

"""``is_element_property`` and ``get_element_property`` as fullrmc calls
them (``Constraints/PairDistributionConstraints.py:599``,
``Core/Collection.py:106-120``): a weighting name is valid when it is one of
the element properties fullrmc's documentation lists, and an element's
property comes from a small table (atomic numbers of a few elements).
Tests that need exact weights pass ``atomsWeight`` explicitly; fullrmc still
evaluates the table lookup as the default of ``dict.get``."""

_PROPERTIES = ("atomicNumber", "neutronCohb", "neutronIncohb", "neutronCohXs", "neutronIncohXs", "atomicWeight",
               "covalentRadius", "atomicFormFactor")

_ATOMIC_NUMBER = {"h": 1, "c": 6, "n": 7, "o": 8, "si": 14, "ti": 22, "fe": 26, "ni": 28, "cu": 29, "zr": 40}


def is_element_property(prop):
    return prop in _PROPERTIES


def get_element_property(element, prop):
    if prop == "atomicNumber":
        return _ATOMIC_NUMBER.get(str(element).lower())
    return None

"""Units and masses with the reference's API (pyvibdmc/simulation_utilities/Constants.py).

The conversion factors and the element table are data that must be identical
to the reference's for unit parity; the table keeps the reference's key order
because ``get_atomic_num`` is the 1-based position in it (Constants.py:41-47).
"""
__all__ = ["Constants", "get_atomic_num", "get_atomic_string"]

# Element masses in amu, in the reference's key order (first 20 entries of Constants.py:3-38).
_MASSES = [("H", 1.00782503), ("D", 2.01410178), ("T", 3.01604928), ("He", 4.00260325), ("Li", 7.01600344),
           ("Be", 9.01218306), ("B", 11.00930536), ("C", 12.0), ("N", 14.003074), ("O", 15.99491462),
           ("F", 18.99840316), ("Ne", 19.99244018), ("Na", 22.98976928), ("Mg", 23.9850417),
           ("Al", 26.98153853), ("Si", 27.97692653), ("P", 30.973762), ("S", 31.97207117),
           ("Cl", 34.96885268), ("Ar", 39.96238312)]
MASS_AMU = dict(_MASSES)
_SYMBOLS = [s for s, _ in _MASSES]


def get_atomic_num(atms):
    """1-based position of each symbol in the element table (Constants.py:41-47)."""
    return [_SYMBOLS.index(a) + 1 for a in atms]


def get_atomic_string(atomic_num):
    if not isinstance(atomic_num, list):
        atomic_num = [atomic_num]
    return [_SYMBOLS[a] for a in atomic_num]


class Constants:
    """Energy, length and mass conversions to/from atomic units (Constants.py:60-119)."""
    atomic_units = {
        "wavenumbers": 4.556335281212229e-6,
        "angstroms": 1 / 0.529177,
        "amu": 1.000000000000000000 / 6.02213670000e23 / 9.10938970000e-28,
    }

    @classmethod
    def convert(cls, val, unit, to_AU=True):
        vv = cls.atomic_units[unit]
        return (val * vv) if to_AU else (val / vv)

    @classmethod
    def mass(cls, atom, to_AU=True):
        m = MASS_AMU[atom]
        return cls.convert(m, "amu") if to_AU else m

    @classmethod
    def reduced_mass(cls, atoms, to_AU=True):
        a, b = atoms.split("-")
        m1, m2 = MASS_AMU[a], MASS_AMU[b]
        if to_AU:
            m1, m2 = cls.convert(m1, "amu"), cls.convert(m2, "amu")
        return m1 * m2 / (m1 + m2)

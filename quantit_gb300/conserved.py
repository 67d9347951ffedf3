"""Conserved quantities: U(1) (``Z``), Z(N) (``C<N>``) and their products.

Mirrors ``quantit.conserved`` (python_binding/conserved.cpp:21-60) and the C++
group classes (include/Conserved/quantity.h).  A ``quantity`` is a tuple of
int16 values with a tuple of moduli (0 for a U(1) factor).
"""


def _wrap16(v):
    return ((int(v) + 32768) % 65536) - 32768


def _make_c(v, n):
    # conserved::C<N>(int16) constructor, include/Conserved/quantity.h:96
    v = int(v)
    r = abs(v) % n
    if v < 0:
        r = -r
    return ((int(v != -n) * int(v < 0)) * n + r) & 0xFFFF


class quantity:
    __slots__ = ("values", "mods")

    def __init__(self, values=(0,), mods=(0,)):
        mods = tuple(int(m) for m in mods)
        self.mods = mods
        self.values = tuple(_make_c(v, m) if m else _wrap16(v) for v, m in zip(values, mods))

    @classmethod
    def _raw(cls, values, mods):
        q = cls.__new__(cls)
        q.values = tuple(values)
        q.mods = tuple(mods)
        return q

    def __mul__(self, other):
        """Group operation (QuantiT writes it as a product)."""
        self._same(other)
        return quantity._raw(tuple(((a + b) % m) if m else _wrap16(a + b)
                                   for a, b, m in zip(self.values, other.values, self.mods)), self.mods)

    __add__ = __mul__

    def inv(self):
        return quantity._raw(tuple((((m - a) if a else 0) if m else _wrap16(-a))
                                   for a, m in zip(self.values, self.mods)), self.mods)

    def neutral(self):
        return quantity._raw(tuple(0 for _ in self.mods), self.mods)

    def _same(self, other):
        if self.mods != other.mods:
            raise TypeError("conserved quantities of different groups")

    def __eq__(self, other):
        return isinstance(other, quantity) and self.mods == other.mods and self.values == other.values

    def __ne__(self, other):
        return not self == other

    def __lt__(self, other):
        self._same(other)
        return self.values < other.values

    def __gt__(self, other):
        self._same(other)
        return self.values > other.values

    def __hash__(self):
        return hash((self.values, self.mods))

    def __repr__(self):
        parts = [f"Z({v})" if m == 0 else f"C<{m}>({v})" for v, m in zip(self.values, self.mods)]
        return "quantity(" + ",".join(parts) + ")"


def Z(x):
    return quantity((x,), (0,))


def C(n):
    def make(x):
        return quantity((x,), (n,))
    return make


C2, C3, C4, C5, C6 = C(2), C(3), C(4), C(5), C(6)


def ZZ(x, y):
    return quantity((x, y), (0, 0))


def ZC(n):
    def make(x, z):
        return quantity((x, z), (0, n))
    return make


ZC2, ZC3, ZC4, ZC5, ZC6 = ZC(2), ZC(3), ZC(4), ZC(5), ZC(6)


def ZZC(n):
    def make(x, y, z):
        return quantity((x, y, z), (0, 0, n))
    return make


ZZC2, ZZC3, ZZC4, ZZC5, ZZC6 = ZZC(2), ZZC(3), ZZC(4), ZZC(5), ZZC(6)

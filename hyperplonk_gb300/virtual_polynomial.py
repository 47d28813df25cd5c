"""VirtualPolynomial: sum of coefficient-weighted products of shared MLE handles.

Host metadata only, restating backend/src/virtual_polynomial.rs:44-235 of the
reference: `products` is a list of (coefficient, [factor index]) and
`flattened_ml_extensions()` holds the distinct factor handles in
first-insertion order, deduplicated by handle identity (`id()`), never by
contents.  Coefficients are canonical Fr integers.
"""
from __future__ import annotations

from dataclasses import dataclass

from .errors import InvalidParameters

R_MODULUS = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


@dataclass
class VPAuxInfo:
    """max_degree and num_variables (virtual_polynomial.rs:76-87).  Its
    canonical serialization is max_degree then num_variables, u64 LE each."""
    max_degree: int
    num_variables: int

    def to_bytes(self) -> bytes:
        return self.max_degree.to_bytes(8, "little") + self.num_variables.to_bytes(8, "little")


class VirtualPolynomial:
    def __init__(self, num_variables: int):
        self.aux_info = VPAuxInfo(0, num_variables)
        self.products: list[tuple[int, list[int]]] = []
        self._flattened: list = []
        self._lookup: dict = {}

    def flattened_ml_extensions(self) -> list:
        return list(self._flattened)

    @classmethod
    def new_from_mle(cls, mle, coefficient: int) -> "VirtualPolynomial":
        vp = cls(mle.num_vars)
        vp.aux_info.max_degree = 1
        vp._flattened = [mle]
        vp._lookup = {mle.id(): 0}
        vp.products = [(coefficient % R_MODULUS, [0])]
        return vp

    def clone(self) -> "VirtualPolynomial":
        vp = VirtualPolynomial(self.aux_info.num_variables)
        vp.aux_info = VPAuxInfo(self.aux_info.max_degree, self.aux_info.num_variables)
        vp.products = [(c, list(ix)) for c, ix in self.products]
        vp._flattened = list(self._flattened)
        vp._lookup = dict(self._lookup)
        return vp

    def add_mle_list(self, mle_list, coefficient: int) -> None:
        """virtual_polynomial.rs:154-192: error (state unchanged) on an empty
        list or a factor of the wrong dimension."""
        mles = list(mle_list)
        if not mles:
            raise InvalidParameters("input mle_list is empty")
        for m in mles:
            if m.num_vars != self.aux_info.num_variables:
                raise InvalidParameters(
                    f"product has a multiplicand with wrong number of variables {m.num_vars} vs "
                    f"{self.aux_info.num_variables}")
        self.aux_info.max_degree = max(self.aux_info.max_degree, len(mles))
        indexed = []
        for m in mles:
            key = m.id()
            if key in self._lookup:
                indexed.append(self._lookup[key])
            else:
                self._lookup[key] = len(self._flattened)
                self._flattened.append(m)
                indexed.append(self._lookup[key])
        self.products.append((coefficient % R_MODULUS, indexed))

    def mul_by_mle(self, mle, coefficient: int) -> None:
        """virtual_polynomial.rs:199-234."""
        if mle.num_vars != self.aux_info.num_variables:
            raise InvalidParameters(
                f"product has a multiplicand with wrong number of variables {mle.num_vars} vs "
                f"{self.aux_info.num_variables}")
        key = mle.id()
        if key in self._lookup:
            idx = self._lookup[key]
        else:
            idx = len(self._flattened)
            self._lookup[key] = idx
            self._flattened.append(mle)
        self.products = [((c * coefficient) % R_MODULUS, ix + [idx]) for c, ix in self.products]
        self.aux_info.max_degree += 1

    def __add__(self, other: "VirtualPolynomial") -> "VirtualPolynomial":
        res = self.clone()
        for c, ix in other.products:
            res.add_mle_list([other._flattened[i] for i in ix], c)
        return res

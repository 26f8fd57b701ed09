"""Registration of the GB300 session as a dmrgpy backend.

dmrgpy picks its session module with ``cppext.get_backend(version)``
(``cppext.py:38-59``), which caches modules in ``cppext._backends``; about
64 call sites then gate on ``itensor_version in (2, 3, "python")``
(``sites.py:20``, ``mode.py:27``, ``groundstate.py:89,104``, ...).  The
backend tags below are ``str`` values that compare equal to ``"python"``
(so every such gate routes them exactly like the python backend) while
hashing to their own values, so ``get_backend(tag)`` returns the GB300
session.
"""
import sys


class _BackendTag(str):
    def __new__(cls, name="gb300", precision="fp64"):
        tag = str.__new__(cls, name)
        tag.precision = precision
        return tag

    def __eq__(self, other):
        if isinstance(other, str) and str.__eq__(other, "python"):
            return True
        return str.__eq__(self, other)

    def __ne__(self, other):
        return not self.__eq__(other)

    def __hash__(self):
        return str.__hash__(self)


# FP64 contractions (the reference's arithmetic) and split-TF32 contractions
# with FP64 reductions and truncation decisions
BACKEND_TAG = _BackendTag("gb300", "fp64")
BACKEND_TAG_TF32 = _BackendTag("gb300-tf32", "tf32x3")


class _SessionModule:
    """What ``cppext.get_backend(tag)`` returns: an object whose ``Chain``
    is the session class (dmrgpy calls ``get_backend(V).Chain(sites)``)."""

    def __init__(self, precision):
        from .session import session_class
        self.Chain = session_class(precision)


def register(precision="fp64"):
    """Insert the GB300 session into dmrgpy's backend registry and return the
    tag to pass as ``itensor_version`` (``precision`` "fp64" or "tf32x3").
    The session is a subclass of dmrgpy's python-backend session
    (:mod:`.session`), so every method and handle dmrgpy's glue uses keeps
    working; the sweeps run on the GPU."""
    from dmrgpy import cppext  # requires dmrgpy
    tag = BACKEND_TAG if precision == "fp64" else BACKEND_TAG_TF32
    if tag.precision != precision:
        raise ValueError("precision must be 'fp64' or 'tf32x3'")
    cppext._backends[tag] = _SessionModule(precision)
    return tag


def setup_gb300(many_body_chain, precision="fp64"):
    """Switch an existing dmrgpy chain object to the GB300 backend (the
    counterpart of ``Many_Body_Chain.setup_python``, manybodychain.py:230-235)."""
    tag = register(precision)
    from dmrgpy import cppext
    many_body_chain.itensor_version = tag
    many_body_chain._session = cppext.get_backend(tag).Chain(many_body_chain.sites)
    return many_body_chain


if __name__ == "__main__":  # pragma: no cover
    sys.exit(0)

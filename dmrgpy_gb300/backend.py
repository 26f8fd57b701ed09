"""Registration of the GB300 session as a dmrgpy backend.

dmrgpy picks its session module with ``cppext.get_backend(version)``
(``cppext.py:38-59``), which caches modules in ``cppext._backends``; about
64 call sites then gate on ``itensor_version in (2, 3, "python")``
(``sites.py:20``, ``mode.py:27``, ``groundstate.py:89,104``, ...).  The
backend tag below is a ``str`` that compares equal to ``"python"`` (so every
such gate routes it exactly like the python backend) while hashing to its
own value, so ``get_backend(tag)`` returns this module.
"""
import sys


class _BackendTag(str):
    def __new__(cls):
        return str.__new__(cls, "gb300")

    def __eq__(self, other):
        if isinstance(other, str) and str.__eq__(other, "python"):
            return True
        return str.__eq__(self, other)

    def __ne__(self, other):
        return not self.__eq__(other)

    def __hash__(self):
        return str.__hash__(self)


BACKEND_TAG = _BackendTag()


def register():
    """Insert this package's session module into dmrgpy's backend registry
    and return the tag to pass as ``itensor_version``."""
    from dmrgpy import cppext  # requires dmrgpy
    from . import chain as _chain_mod
    cppext._backends[BACKEND_TAG] = _chain_mod
    return BACKEND_TAG


def setup_gb300(many_body_chain):
    """Switch an existing dmrgpy chain object to the GB300 backend (the
    counterpart of ``Many_Body_Chain.setup_python``, manybodychain.py:230-235)."""
    tag = register()
    many_body_chain.itensor_version = tag
    from . import chain as _chain_mod
    many_body_chain._session = _chain_mod.Chain(many_body_chain.sites)
    return many_body_chain


if __name__ == "__main__":  # pragma: no cover
    sys.exit(0)

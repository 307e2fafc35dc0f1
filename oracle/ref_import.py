"""Import the reference tskit Python package for fixture generation.

Test infrastructure only (never imported by the product).  The reference's
CPython extension ``_tskit`` is compiled by ``make -C oracle ref`` into
``oracle/_ref/``; the reference's pure-Python package is read from the
reference checkout, whose location is given by ``TSKIT_REFERENCE`` or else
by the source location that build recorded in ``oracle/_ref/SOURCE``.  The package
imports ``jsonschema`` at module import; ``oracle/shim`` supplies a no-op
stand-in because jsonschema is not installed.
"""
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))


def reference_root():
    """The reference checkout: ``TSKIT_REFERENCE``, else the one the
    ``oracle/_ref`` build was made from (None when neither is known)."""
    root = os.environ.get("TSKIT_REFERENCE")
    if root:
        return root
    try:
        with open(os.path.join(_HERE, "_ref", "SOURCE")) as f:
            return f.read().strip() or None
    except OSError:
        return None


def available():
    root = reference_root()
    if root is None:
        return False
    return os.path.isdir(os.path.join(root, "python", "tskit")) and any(
        f.startswith("_tskit") for f in os.listdir(os.path.join(_HERE, "_ref"))
    ) if os.path.isdir(os.path.join(_HERE, "_ref")) else False


def import_tskit():
    """Return the reference ``tskit`` module (raises ImportError if absent)."""
    if not available():
        raise ImportError("reference tskit not built: run `make -C oracle ref`")
    for p in (os.path.join(_HERE, "_ref"), os.path.join(_HERE, "shim"),
              os.path.join(reference_root(), "python")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import tskit  # noqa: E402

    return tskit

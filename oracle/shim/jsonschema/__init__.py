"""Minimal stand-in for the ``jsonschema`` package (not installed here).

Test infrastructure only: it lets the reference ``tskit`` Python package be
imported in order to generate golden fixtures.  Metadata validation is a
no-op, which is irrelevant for the statistics path (it never touches
metadata).  The reference needs ``validators.extend``, a ``Draft7Validator``
class carrying a ``META_SCHEMA`` dict with ``definitions`` and ``properties``
keys, ``ValidationError``/``SchemaError`` and the private ``_validators`` /
``_keywords`` hooks (tskit/metadata.py:41-81, 137-153, 342-414).
"""
from . import exceptions, validators  # noqa: F401
from .exceptions import SchemaError, ValidationError  # noqa: F401
from . import _validators, _keywords  # noqa: F401

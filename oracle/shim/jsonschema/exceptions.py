"""Exception names used by the reference package."""


class ValidationError(Exception):
    pass


class SchemaError(Exception):
    pass

"""No-op validator classes with the attributes the reference reads."""
import copy


class _Validator:
    META_SCHEMA = {
        "$schema": "http://json-schema.org/draft-07/schema#",
        "definitions": {},
        "properties": {"type": {}},
        "type": ["object", "boolean"],
    }
    VALIDATORS = {}

    def __init__(self, schema, *args, **kwargs):
        self.schema = schema

    @classmethod
    def check_schema(cls, schema):
        return None

    def validate(self, instance, *args, **kwargs):
        return None

    def iter_errors(self, instance, *args, **kwargs):
        return iter(())

    def is_valid(self, instance, *args, **kwargs):
        return True


class Draft7Validator(_Validator):
    pass


def extend(validator, validators=(), version=None, type_checker=None, **kwargs):
    new = type("ExtendedValidator", (validator,), {})
    new.META_SCHEMA = copy.deepcopy(validator.META_SCHEMA)
    new.VALIDATORS = dict(getattr(validator, "VALIDATORS", {}))
    new.VALIDATORS.update(dict(validators))
    return new

def type(validator, types, instance, schema):  # noqa: A001
    return iter(())


def properties(validator, properties, instance, schema):
    return iter(())


def required(validator, required, instance, schema):
    return iter(())

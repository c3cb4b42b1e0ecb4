"""Pytree registration is a no-op: jit is the identity, so nothing is flattened."""


def register_pytree_node_class(cls):
    return cls

"""Stand-in for PyYAML exposing only what the reference registers at import."""


class _Registry:
    @classmethod
    def add_representer(cls, *a, **k):
        pass

    @classmethod
    def add_constructor(cls, *a, **k):
        pass

    @classmethod
    def add_implicit_resolver(cls, *a, **k):
        pass


class SafeLoader(_Registry):
    pass


class SafeDumper(_Registry):
    pass


class Loader(_Registry):
    pass


class Dumper(_Registry):
    pass


class Node:
    pass


class ScalarNode(Node):
    pass


def safe_load(*a, **k):
    raise RuntimeError("yaml stand-in: parsing unavailable")


def load(*a, **k):
    raise RuntimeError("yaml stand-in: parsing unavailable")


def dump(*a, **k):
    return ""


safe_dump = dump


def add_representer(*a, **k):
    pass


def add_constructor(*a, **k):
    pass


def add_implicit_resolver(*a, **k):
    pass

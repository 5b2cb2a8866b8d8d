"""Stand-ins for warp.utils names XLB imports at module scope."""


class ScopedTimer:
    def __init__(self, *a, **k):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

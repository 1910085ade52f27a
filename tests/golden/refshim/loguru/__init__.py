"""No-op stand-in for ``loguru`` (absent here) so the unmodified reference
torchquad can be imported to record golden fixtures.  Test infrastructure."""


class _Logger:
    def opt(self, *args, **kwargs):
        return self

    def _noop(self, *args, **kwargs):
        return None

    debug = info = warning = error = critical = trace = success = exception = _noop
    remove = enable = disable = level = _noop

    def add(self, *args, **kwargs):
        return 0


logger = _Logger()

"""ORACLE test infrastructure: no-op plotting calls (see matplotlib/__init__.py)."""


def _noop(*a, **k):
    return None


plot = yscale = legend = show = figure = savefig = ylim = xlabel = ylabel = title = close = _noop

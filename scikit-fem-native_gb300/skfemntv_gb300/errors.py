"""Exception types of the public API (same names and bases as the reference:
python/skfemntv/_errors.py:4, python/skfemntv/preflight.py:96)."""


class UnsupportedNativeForm(NotImplementedError):
    """A form or element the GPU backend does not assemble."""

"""Single source of the package version (the reference API version it implements)."""

__version__ = "0.2.0"

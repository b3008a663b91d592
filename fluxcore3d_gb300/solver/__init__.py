"""Reference-compatible solver modules (see the package docstring)."""

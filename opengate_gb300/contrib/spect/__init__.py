"""SPECT head and digitizer helpers (opengate/contrib/spect counterparts)."""

"""Helpers that build common set-ups on the opengate-shaped API (opengate/contrib counterparts)."""

"""Integrators with the reference torchquad class names (torch backend only)."""

"""Configuration helpers with the reference's names (torchquad/utils)."""

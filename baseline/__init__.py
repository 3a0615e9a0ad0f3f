"""Comparators that bench.py times beside this library: the reference's own
pytorch GPU path (plain_gpu).  Not part of the library."""

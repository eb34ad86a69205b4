"""Cython binding of the engine (NCVisWrapper), built by build.py."""

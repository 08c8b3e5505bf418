"""Stand-in for numba.typed (see __init__.py)."""
List = list

"""Examples: a C++ host program (poisson_cube.cpp) and a Python driver (poisson_msh.py)."""

"""CPU oracle of the null-collision step: test infrastructure only (see oracle.cpp)."""

"""CPU oracle of the alignment path -- test infrastructure only (see oracle.h)."""

"""GB300-native lattice evolution (Abelian-Higgs and Moore models) behind a C ABI."""

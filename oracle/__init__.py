"""CPU oracle of the SpecMC time step (test infrastructure; see specmc_oracle)."""

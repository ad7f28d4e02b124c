"""CPU oracle for the HDBSCAN fit core: test infrastructure, never part of the product path."""

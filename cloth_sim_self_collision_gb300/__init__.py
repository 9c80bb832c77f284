"""GB300-native FEM cloth step with self-collision (the self_contact_sparse path)."""

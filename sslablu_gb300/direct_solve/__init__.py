"""Mirror of the upstream package of the same name."""

"""CPU oracle of the PGDG particle-grid path (test infrastructure only)."""

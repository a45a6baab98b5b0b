"""CPU oracle of the channel-flow hot path (test infrastructure only)."""

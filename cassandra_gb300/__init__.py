"""GB300-native Cassandra molecular-energy hot path."""

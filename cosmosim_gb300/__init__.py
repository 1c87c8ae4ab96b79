"""GB300-native gravity/SPH hot path for cosmosim."""

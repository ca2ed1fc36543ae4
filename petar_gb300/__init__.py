"""GB300-native long-range soft-force kernels for PeTar (EP-EP linear-cutoff
gravity, EP-SP quadrupole gravity and the r_search neighbour count) behind the
reference's multi-walk dispatch/retrieve functor pair."""

/* empty: Aztec definitions live in az_aztec.h for the oracle build */

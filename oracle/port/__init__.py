"""Float64 C port of the reference algorithm (test infrastructure only; CPU baseline)."""

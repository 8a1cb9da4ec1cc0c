"""CPU oracle of the reference clustering — test infrastructure only (the
reference results the parity tests compare against, and the CPU baseline);
the product never imports it."""

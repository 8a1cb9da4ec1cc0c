"""CPU oracle of the reference clustering — test infrastructure only (the
parity checker and the CPU baseline); the product never imports it."""

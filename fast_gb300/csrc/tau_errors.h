// Per-thread error message shared by the translation units of the library
// (fast_last_error() returns it).
#pragma once

int ft_fail(int status, const char *fmt, ...);
void ft_clear_error();

// Keep memory freed into the device's default stream-ordered pool for the
// next call of the library (its solves, labellings and area passes
// allocate their scratch from that pool), instead of returning it to the
// driver at every synchronisation.  Applied once per device.
void ft_retain_pool_memory(int device);

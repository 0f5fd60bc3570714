// Per-thread error message shared by the translation units of the library
// (fast_last_error() returns it).
#pragma once

int ft_fail(int status, const char *fmt, ...);
void ft_clear_error();

// Forced into every reference translation unit compiled for the oracle.
// The reference's material files call abs() on floats with only
// <bits/stdc++.h> in scope; on Linux/glibc that binds to int abs(int) and
// truncates |cos| to 0 (Lambert pdf becomes 1e-4/pi). The reference's
// published renders (docs/imgs/hack_cboxb_32spp.jpg: coloured indirect light
// on the walls under ptnee) show the float overload was in effect on the
// author's build, so the oracle makes std::abs(float) visible globally, as a Qt or
// MinGW build does. Only abs is affected: every other libm call on floats
// keeps binding to the C double-precision function, as on a plain Linux build.
#pragma once
#include <cstdlib>
using std::abs;

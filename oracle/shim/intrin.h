// Test infrastructure: the reference's utils.h includes the MSVC header
// <intrin.h>; nothing on the Demo4 step path uses it, so it is empty here.

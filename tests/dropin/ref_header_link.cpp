// Link check of the drop-in: a C++ caller written against the reference's own meshoptimizer.h,
// using its 32-bit entry points and its header-only 16-bit templates (meshopt_simplify<T> and
// meshopt_simplifyWithAttributes<T>, which widen through meshopt_IndexAdapter), built and linked
// with libmeshopt_gb300.so and nothing else. Including this library's header after the
// reference's shows that one translation unit can use both.
#include "meshoptimizer.h"
#include "meshopt_gb300.h"

#include <stdio.h>

int main()
{
	const unsigned int idx[6] = {0, 1, 2, 2, 1, 3};
	const unsigned short idx16[6] = {0, 1, 2, 2, 1, 3};
	const float pos[12] = {0, 0, 0, 1, 0, 0, 0, 1, 0, 1, 1, 0};
	const float attr[4] = {0, 1, 0, 1};
	const float weight = 1.f;
	unsigned int out[6];
	unsigned short out16[6];
	float err = 0;
	size_t a = meshopt_simplify(out, idx, 6, pos, 4, 12, 3, 1e-2f, meshopt_SimplifyLockBorder, &err);
	size_t b = meshopt_simplifyWithAttributes(out, idx, 6, pos, 4, 12, attr, 4, &weight, 1, NULL, 3, 1e-2f, 0, &err);
	size_t c = meshopt_simplify(out16, idx16, 6, pos, 4, 12, 3, 1e-2f, 0, &err);
	size_t d = meshopt_simplifyWithAttributes(out16, idx16, 6, pos, 4, 12, attr, 4, &weight, 1, NULL, 3, 1e-2f, 0, &err);
	float s = meshopt_simplifyScale(pos, 4, 12);
	printf("%zu %zu %zu %zu %g %d\n", a, b, c, d, s, meshoptgpu_getLastStatus());
	return 0;
}

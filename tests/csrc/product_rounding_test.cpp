// ChargePotForce (src/model/forcefield.h:87-146) forms its forces as
// (float)(et2 * (double)d) with et2 a float-valued double: the exact product
// of two floats has at most 48 significant bits, so the double product is
// exact and the conversion rounds once -- the single-precision product,
// subnormals and overflow included.  The reference-order kernels rely on it;
// this checks it on random operands over the whole float range (built with
// -ffp-contract=off).  Exit status 1 on any mismatch.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

static uint32_t bits(float f) {
	uint32_t u;
	std::memcpy(&u, &f, 4);
	return u;
}

static float from_bits(uint32_t u) {
	float f;
	std::memcpy(&f, &u, 4);
	return f;
}

int main(int argc, char** argv) {
	const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
	std::mt19937_64 rng(2024);
	long bad = 0, checked = 0;
	for (long i = 0; i < n; ++i) {
		// any finite float: exponent field 0..254, random sign and fraction
		const auto draw = [&]() {
			return from_bits((uint32_t)(rng() & 0x807fffffu) | (uint32_t)(rng() % 255) << 23);
		};
		const float e = draw(), d = draw();
		const float want = (float)((double)e * (double)d);
		if (bits(e * d) != bits(want)) ++bad;
		++checked;
		const float e2 = 2.f * e;
		if (std::isfinite(e2)) {
			if (bits(e2 * d) != bits((float)(2 * (double)e * (double)d))) ++bad;
			++checked;
		}
	}
	std::printf("%ld products checked, %ld mismatches\n", checked, bad);
	return bad == 0 ? 0 : 1;
}

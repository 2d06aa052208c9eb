// Prints the first draws of the reference pcg wrapper (include/Rand.hpp:249-291)
// for a few seeds, as golden vectors for the project's PCG32.  Test infrastructure.
#include <cstdio>
#include "Rand.hpp"
int main() {
    const unsigned long long seeds[] = {1ULL, 7ULL, 42ULL, 123456789ULL, 18446744073709551557ULL};
    for (unsigned long long s : seeds) {
        pcg g;
        g.set_seed(s);
        printf("%llu", s);
        for (int i = 0; i < 16; ++i) printf(" %a", g.doub());
        printf("\n");
    }
    return 0;
}

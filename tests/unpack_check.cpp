// Exhaustive check of mcg_unpack_tsdf against IEEE division (built and run
// by tests/test_unpack_exact.py with -ffp-contract=off).
#include <stdio.h>
#include <string.h>
#include "unpack.h"

int main() {
    int bad = 0;
    for (int t = -32768; t <= 32767; ++t) {
        volatile float a = (float)t;
        volatile float ref = a / 32766.0f;
        float got = mcg_unpack_tsdf(t);
        unsigned int x, y;
        float r = ref;
        memcpy(&x, &got, 4);
        memcpy(&y, &r, 4);
        if (x != y) {
            if (bad < 5) printf("mismatch t=%d got=%a ref=%a\n", t, got, r);
            ++bad;
        }
    }
    printf("%d mismatches\n", bad);
    return bad != 0;
}

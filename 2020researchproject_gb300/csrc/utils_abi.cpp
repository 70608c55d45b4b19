// Helper functions the reference exports from src/utils.c and its case
// drivers call (fopen_check in src/main.c:67-74 and building.c:35; the
// others for drivers that post-process fields).  Declared in
// include/utils.h with the reference's names and meanings.
#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "utils.h"

extern "C" {

FILE *fopen_check(const char *filename, const char *modes) {
    FILE *fp = std::fopen(filename, modes);
    if (!fp) {
        std::fprintf(stderr, "error: cannot open file \"%s\"\n", filename);
        std::exit(255);  // the reference aborts its MPI job with -1
    }
    return fp;
}

double sq(const double x) { return x * x; }

int lower_bound(const int len, const double arr[], const double val) {
    return len <= 0 ? 0 : (int)(std::lower_bound(arr, arr + len, val) - arr);
}

int upper_bound(const int len, const double arr[], const double val) {
    return len <= 0 ? 0 : (int)(std::upper_bound(arr, arr + len, val) - arr);
}

int dir_to_idx(IBMSolverDirection dir) {
    for (int b = 0; b < 6; b++)
        if (dir == (IBMSolverDirection)(1 << b)) return b;
    return -1;
}

int divceil(int a, int b) { return (a + b - 1) / b; }

}  // extern "C"

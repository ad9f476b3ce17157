// CPU check of the screened assignment's candidate-list guard (screen.cuh):
// well-formed lists are used as written; a count out of range, an entry outside
// [0, k), or entries out of ascending order mean "evaluate every centroid".
// Built and run by tests/test_screen_list.py (no GPU).
#include <cstdio>

#include "screen.cuh"

using tc::screen_list_len;
using tc::SCREEN_CAP;

static int fails = 0;
static void expect(int got, int want, const char* what) {
    if (got != want) {
        printf("FAIL %s: got %d want %d\n", what, got, want);
        ++fails;
    }
}

int main() {
    int l[SCREEN_CAP] = {0, 3, 5, 6, 9, 10, 20, 31};
    expect(screen_list_len(l, 1, 32), 1, "one candidate");
    expect(screen_list_len(l, 8, 32), 8, "full list");
    expect(screen_list_len(l, -1, 32), -1, "all centroids");
    expect(screen_list_len(l, 0, 32), -1, "empty list");
    expect(screen_list_len(l, 9, 32), -1, "count above the cap");
    expect(screen_list_len(l, 0x7fffffff, 32), -1, "count never written (large)");
    expect(screen_list_len(l, -17, 32), -1, "count never written (negative)");
    expect(screen_list_len(l, 8, 31), -1, "entry >= k (stale list of a larger k)");
    expect(screen_list_len(l, 7, 31), 7, "entries below k");
    int neg[3] = {-1, 2, 4};
    expect(screen_list_len(neg, 3, 8), -1, "negative entry");
    int dup[3] = {1, 1, 4};
    expect(screen_list_len(dup, 3, 8), -1, "repeated entry");
    int desc[3] = {4, 2, 1};
    expect(screen_list_len(desc, 3, 8), -1, "descending entries");
    if (fails == 0) printf("ALL OK\n");
    return fails ? 1 : 0;
}

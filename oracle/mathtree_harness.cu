// Test infrastructure: evaluates VXA formula token lists with the reference's own
// evaluator, VX3_MathTree::eval (Voxelyze3/src/Utils/VX3_MathTree.h:50-192), compiled as
// host code from the reference's header (recipe: oracle/Makefile, target `mathtree`;
// output in oracle/_ref/).  Used only to generate the golden values of
// tests/golden/formulas.json.
//
// Input (stdin), one case per line:  T op_0 value_0 ... op_{T-1} value_{T-1} N v_0 ... v_{9N-1}
//   (token ops are the enum values of VX3_MathTreeOperator; each variable set is x, y, z,
//   hit, t, angle, closeness, numClosePairs, num_voxel)
// Output (stdout), one line per case: the N results with %.17g, or "error" where eval throws.
#include <cstdio>
#include <vector>

#include "VX3_MathTree.h"

int main() {
    int T;
    while (std::scanf("%d", &T) == 1) {
        std::vector<VX3_MathTreeToken> buf(1024);
        for (int i = 0; i < T && i < 1024; i++) {
            int op;
            double v;
            if (std::scanf("%d %lf", &op, &v) != 2) return 1;
            buf[i].set((VX3_MathTreeOperator)op, v);
        }
        int N;
        if (std::scanf("%d", &N) != 1) return 1;
        for (int k = 0; k < N; k++) {
            double v[9];
            for (int j = 0; j < 9; j++)
                if (std::scanf("%lf", &v[j]) != 1) return 1;
            try {
                const double r = VX3_MathTree::eval(v[0], v[1], v[2], v[3], v[4], v[5], v[6], (int)v[7], (int)v[8], buf.data());
                std::printf("%s%.17g", k ? " " : "", r);
            } catch (...) {
                std::printf("%serror", k ? " " : "");
            }
        }
        std::printf("\n");
        std::fflush(stdout);
    }
    return 0;
}

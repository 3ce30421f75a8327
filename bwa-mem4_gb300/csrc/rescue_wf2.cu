// rescue_wf2.cu -- launches of the paired register wavefront (rescue_wf2.cuh): two rescue jobs
// per group of 4, 8 or 16 lanes, one in each 16-bit lane of the registers.  This unit builds the
// kernels of scorings whose gap opens agree (o_del + e_del == o_ins + e_ins, bwa's default);
// rescue_wf2a.cu the others.
#include "rescue_wf2.cuh"

namespace bwacuda {

namespace wf2 {

cudaError_t launch_sym(const RescueLaunch &Lr, int lanes, int c, int npen)
{
    return launch_shape<true>(Lr, lanes, c, npen);
}

}  // namespace wf2

namespace {

// The scoring suits the paired wavefront when the alphabet is at most bwa's five letters, the N
// row and column hold one value (the profile words cover codes 0..3; a target N row scores that
// value on every real column), and the gap costs are non-negative with o_del + e_del <= 128 (a
// column past the query, scored -128, then never holds a row maximum).
bool pair_scoring_ok(const Scoring &sc, int *npen)
{
    if (sc.m > 5 || sc.o_del < 0 || sc.e_del < 0 || sc.o_ins < 0 || sc.e_ins < 0) return false;
    if (sc.o_del + sc.e_del > 128) return false;
    *npen = 0;
    if (sc.m < 5) return true;
    const int8_t n0 = (int8_t)(sc.prof[0][1] & 0xffu);  // mat[0][4]
    for (int t = 1; t < 5; ++t)
        if ((int8_t)(sc.prof[t][1] & 0xffu) != n0) return false;  // mat[t][4]
    for (int q = 0; q < 4; ++q)
        if ((int8_t)((sc.prof[4][0] >> (8 * q)) & 0xffu) != n0) return false;  // mat[4][q]
    *npen = n0;
    return true;
}

// Columns per lane: the smallest built C with L * C >= need.
template <size_t N>
int pick_c(const int (&cs)[N], int lanes, int need)
{
    for (int c : cs)
        if (lanes * c >= need) return c;
    return 0;
}

}  // namespace

cudaError_t rescue_wf2_launch(const RescueLaunch &Lr, int qcap, int lanes, int *cols)
{
    *cols = 0;
    int npen = 0;
    if (!pair_scoring_ok(Lr.sc, &npen)) return cudaSuccess;
    // the launch's queries pad to qcap - 16 columns at most (the callers size qcap with 16 spare)
    int need = qcap - 16;
    if (need < 16) need = 16;
    if (need > 256) need = 256;
    int L = lanes == 16 ? 16 : (lanes == 4 ? 4 : 8);
    int c = L == 16 ? pick_c(wf2::C16, 16, need) : (L == 4 ? pick_c(wf2::C4, 4, need) : pick_c(wf2::C8, 8, need));
    if (c == 0 && L == 4) {  // queries past 4-lane groups' columns: 8-lane groups
        L = 8;
        c = pick_c(wf2::C8, 8, need);
    }
    if (c == 0) return cudaSuccess;
    *cols = L * c;
    const bool sym = Lr.sc.o_del + Lr.sc.e_del == Lr.sc.o_ins + Lr.sc.e_ins;
    return sym ? wf2::launch_sym(Lr, L, c, npen) : wf2::launch_asym(Lr, L, c, npen);
}

}  // namespace bwacuda

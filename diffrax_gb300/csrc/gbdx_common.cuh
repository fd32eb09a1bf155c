// gbdx_common.cuh -- device building blocks of the batched integrator.
//
// Everything a trajectory needs lives in registers: the state y, the RK stage
// increments k_i, the FSAL vector, the PID history and the time grid.  Time t
// and step size dt are FP64; the state, stages and error norm are in the state
// dtype T (FP32 or FP64).  Semantics follow Diffrax v0.7.2:
//   loop body ........ diffrax/_integrate.py:365-662
//   ERK step ......... diffrax/_solver/runge_kutta.py:446-1203
//   PID .............. diffrax/_step_size_controller/pid.py:394-567
//   constant ......... diffrax/_step_size_controller/constant.py:59-104
//   interpolants ..... diffrax/_solver/tsit5.py:103-156,
//                      diffrax/_local_interpolation.py:29-139
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "../../include/gbdx.h"

namespace gbdx {

// ---------------------------------------------------------------------------
// Butcher tableaus (published method constants; the reference stores the same
// numbers in tsit5.py:18-100, dopri5.py:11-33, heun.py:12-17, euler.py).
// ---------------------------------------------------------------------------
template <int SOLVER>
struct Tab;

template <>
struct Tab<GBDX_TSIT5> {
  static constexpr int S = 7;
  static constexpr bool FSAL = true, SSAL = true;
  static constexpr int ORDER = 5;
  static constexpr double STRONG_ORDER = 0.0;
  __host__ __device__ static constexpr double bs(int j) {
    constexpr double v[7] = {
        0.9646076681806522951816731316512876333711995238157997181903319145764851595234062815396e-1,
        1.0 / 100,
        0.4798896504144995747752495322905965199130404621990332488332634944254542060153074523509,
        1.379008574103741893192274821856872770756462643091360525934940067397245698027561293331,
        -3.290069515436080679901047585711363850115683290894936158531296799594813811049925401677,
        2.324710524099773982415355918398765796109060233222962411944060046314465391054716027841,
        0.0};
    return v[j];
  }
  __host__ __device__ static constexpr double c(int i) {
    constexpr double v[7] = {
        0.0, 161.0 / 1000, 327.0 / 1000, 9.0 / 10,
        0.9800255409045096857298102862870245954942137979563024768854764293221195950761080302604,
        1.0, 1.0};
    return v[i];
  }
  __host__ __device__ static constexpr double a(int i, int j) {
    constexpr double v[7][6] = {
        {0, 0, 0, 0, 0, 0},
        {161.0 / 1000, 0, 0, 0, 0, 0},
        {-0.8480655492356988544426874250230774675121177393430391537369234245294192976164141156943e-2,
         0.3354806554923569885444268742502307746751211773934303915373692342452941929761641411569, 0,
         0, 0, 0},
        {2.897153057105493432130432594192938764924887287701866490314866693455023795137503079289,
         -6.359448489975074843148159912383825625952700647415626703305928850207288721235210244366,
         4.362295432869581411017727318190886861027813359713760212991062156752264926097707165077, 0,
         0, 0},
        {5.325864828439256604428877920840511317836476253097040101202360397727981648835607691791,
         -11.74888356406282787774717033978577296188744178259862899288666928009020615663593781589,
         7.495539342889836208304604784564358155658679161518186721010132816213648793440552049753,
         -0.9249506636175524925650207933207191611349983406029535244034750452930469056411389539635e-1,
         0, 0},
        {5.861455442946420028659251486982647890394337666164814434818157239052507339770711679748,
         -12.92096931784710929170611868178335939541780751955743459166312250439928519268343184452,
         8.159367898576158643180400794539253485181918321135053305748355423955009222648673734986,
         -0.7158497328140099722453054252582973869127213147363544882721139659546372402303777878835e-1,
         -0.2826905039406838290900305721271224146717633626879770007617876201276764571291579142206e-1,
         0},
        {0.9646076681806522951816731316512876333711995238157997181903319145764851595234062815396e-1,
         1.0 / 100,
         0.4798896504144995747752495322905965199130404621990332488332634944254542060153074523509,
         1.379008574103741893192274821856872770756462643091360525934940067397245698027561293331,
         -3.290069515436080679901047585711363850115683290894936158531296799594813811049925401677,
         2.324710524099773982415355918398765796109060233222962411944060046314465391054716027841}};
    return v[i][j];
  }
  __host__ __device__ static constexpr double b(int j) { return bs(j); }
  __host__ __device__ static constexpr double e(int j) {
    constexpr double v[7] = {
        0.9646076681806522951816731316512876333711995238157997181903319145764851595234062815396e-1 -
            0.9468075576583945807478876255758922856117527357724631226139574065785592789071067303271e-1,
        1.0 / 100 -
            0.9183565540343253096776363936645313759813746240984095238905939532922955247253608687270e-2,
        0.4798896504144995747752495322905965199130404621990332488332634944254542060153074523509 -
            0.4877705284247615707855642599631228241516691959761363774365216240304071651579571959813,
        1.379008574103741893192274821856872770756462643091360525934940067397245698027561293331 -
            1.234297566930478985655109673884237654035539930748192848315425833500484878378061439761,
        -3.290069515436080679901047585711363850115683290894936158531296799594813811049925401677 +
            2.707712349983525454881109975059321670689605166938197378763992255714444407154902012702,
        2.324710524099773982415355918398765796109060233222962411944060046314465391054716027841 -
            1.866628418170587035753719399566211498666255505244122593996591602841258328965767580089,
        -1.0 / 66};
    return v[j];
  }
};

template <>
struct Tab<GBDX_DOPRI5> {
  static constexpr int S = 7;
  static constexpr bool FSAL = true, SSAL = true;
  static constexpr int ORDER = 5;
  static constexpr double STRONG_ORDER = 0.0;
  __host__ __device__ static constexpr double c(int i) {
    constexpr double v[7] = {0.0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1.0, 1.0};
    return v[i];
  }
  __host__ __device__ static constexpr double a(int i, int j) {
    constexpr double v[7][6] = {
        {0, 0, 0, 0, 0, 0},
        {1.0 / 5, 0, 0, 0, 0, 0},
        {3.0 / 40, 9.0 / 40, 0, 0, 0, 0},
        {44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0, 0},
        {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0, 0},
        {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656, 0},
        {35.0 / 384, 0.0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84}};
    return v[i][j];
  }
  __host__ __device__ static constexpr double b(int j) {
    constexpr double v[7] = {35.0 / 384, 0.0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784,
                             11.0 / 84, 0.0};
    return v[j];
  }
  __host__ __device__ static constexpr double e(int j) {
    constexpr double v[7] = {35.0 / 384 - 1951.0 / 21600, 0.0, 500.0 / 1113 - 22642.0 / 50085,
                             125.0 / 192 - 451.0 / 720, -2187.0 / 6784 - -12231.0 / 42400,
                             11.0 / 84 - 649.0 / 6300, -1.0 / 60.0};
    return v[j];
  }
  // Dense-output midpoint weights (dopri5.py:36-47).
  __host__ __device__ static constexpr double cmid(int j) {
    constexpr double v[7] = {6025192743.0 / 30085553152.0 / 2, 0.0,
                             51252292925.0 / 65400821598.0 / 2,
                             -2691868925.0 / 45128329728.0 / 2,
                             187940372067.0 / 1594534317056.0 / 2,
                             -1776094331.0 / 19743644256.0 / 2, 11237099.0 / 235043384.0 / 2};
    return v[j];
  }
};

template <>
struct Tab<GBDX_HEUN> {
  static constexpr int S = 2;
  static constexpr bool FSAL = false, SSAL = false;
  static constexpr int ORDER = 2;
  static constexpr double STRONG_ORDER = 0.5;
  __host__ __device__ static constexpr double c(int i) { return i == 0 ? 0.0 : 1.0; }
  __host__ __device__ static constexpr double a(int i, int j) { return (i == 1 && j == 0) ? 1.0 : 0.0; }
  __host__ __device__ static constexpr double b(int j) { return 0.5; }
  __host__ __device__ static constexpr double e(int j) { return j == 0 ? 0.5 : -0.5; }
};

// The additive-noise stochastic Runge--Kutta tableaus (srk.py
// StochasticButcherTableau with AdditiveCoeffs): the drift rows, and the W
// and H coefficients of each stage (aw, ah) and of the solution (bw, bh).
__host__ __device__ constexpr bool is_srk(int solver) {
  return solver == GBDX_SHARK || solver == GBDX_SRA1 || solver == GBDX_SEA;
}

// ShARK (shark.py:10-35)
template <>
struct Tab<GBDX_SHARK> {
  static constexpr int S = 2;
  static constexpr bool FSAL = false, SSAL = false;
  static constexpr int ORDER = 2;
  static constexpr double STRONG_ORDER = 1.5;
  __host__ __device__ static constexpr double c(int i) { return i == 0 ? 0.0 : 5.0 / 6.0; }
  __host__ __device__ static constexpr double a(int i, int j) {
    return (i == 1 && j == 0) ? 5.0 / 6.0 : 0.0;
  }
  __host__ __device__ static constexpr double b(int j) { return j == 0 ? 0.4 : 0.6; }
  __host__ __device__ static constexpr double e(int j) { return j == 0 ? -0.6 : 0.6; }
  __host__ __device__ static constexpr double aw(int j) { return j == 0 ? 0.0 : 5.0 / 6.0; }
  __host__ __device__ static constexpr double ah(int) { return 1.0; }
  static constexpr double BW = 1.0, BH = 0.0;
};

// SRA1 (sra1.py:10-34; Roessler 2010)
template <>
struct Tab<GBDX_SRA1> {
  static constexpr int S = 2;
  static constexpr bool FSAL = false, SSAL = false;
  static constexpr int ORDER = 2;
  static constexpr double STRONG_ORDER = 1.5;
  __host__ __device__ static constexpr double c(int i) { return i == 0 ? 0.0 : 3.0 / 4.0; }
  __host__ __device__ static constexpr double a(int i, int j) {
    return (i == 1 && j == 0) ? 3.0 / 4.0 : 0.0;
  }
  __host__ __device__ static constexpr double b(int j) { return j == 0 ? 1.0 / 3.0 : 2.0 / 3.0; }
  __host__ __device__ static constexpr double e(int j) { return j == 0 ? -2.0 / 3.0 : 2.0 / 3.0; }
  __host__ __device__ static constexpr double aw(int j) { return j == 0 ? 0.0 : 3.0 / 4.0; }
  __host__ __device__ static constexpr double ah(int j) { return j == 0 ? 0.0 : 1.5; }
  static constexpr double BW = 1.0, BH = 0.0;
};

// SEA, the shifted Euler method (sea.py:10-34): one stage, no error estimate
template <>
struct Tab<GBDX_SEA> {
  static constexpr int S = 1;
  static constexpr bool FSAL = false, SSAL = false;
  static constexpr int ORDER = 1;
  static constexpr double STRONG_ORDER = 1.0;
  __host__ __device__ static constexpr double c(int) { return 0.0; }
  __host__ __device__ static constexpr double a(int, int) { return 0.0; }
  __host__ __device__ static constexpr double b(int) { return 1.0; }
  __host__ __device__ static constexpr double e(int) { return 0.0; }
  __host__ __device__ static constexpr double aw(int) { return 0.5; }
  __host__ __device__ static constexpr double ah(int) { return 1.0; }
  static constexpr double BW = 1.0, BH = 0.0;
};

template <>
struct Tab<GBDX_EULER> {
  static constexpr int S = 1;
  static constexpr bool FSAL = false, SSAL = false;
  static constexpr int ORDER = 1;
  static constexpr double STRONG_ORDER = 0.5;
  __host__ __device__ static constexpr double c(int) { return 0.0; }
  __host__ __device__ static constexpr double a(int, int) { return 0.0; }
  __host__ __device__ static constexpr double b(int) { return 1.0; }
  __host__ __device__ static constexpr double e(int) { return 0.0; }
};


// Dopri8 (dopri8.py:18-189): Prince and Dormand's 8(7) pair with 14 stages,
// FSAL and SSAL (the last stage is evaluated at y1), and the Bogacki--Shampine
// dense output y(theta) = y0 + sum_j theta P_j(theta) k_j (dopri8.py:192-303,
// P_j of degree 5, highest power first).  Published method constants, written
// as the exact rational quotients.
template <>
struct Tab<GBDX_DOPRI8> {
  static constexpr int S = 14;
  static constexpr bool FSAL = true, SSAL = true;
  static constexpr int ORDER = 8;
  static constexpr double STRONG_ORDER = 0.0;
  __host__ __device__ static constexpr double c(int i) {
    constexpr double v[14] = {0.0, (1.0 / 18.0), (1.0 / 12.0), (1.0 / 8.0), (5.0 / 16.0), (3.0 / 8.0), (59.0 / 400.0), (93.0 / 200.0), (5490023248.0 / 9719169821.0), (13.0 / 20.0), (1201146811.0 / 1299019798.0), 1.0, 1.0, 1.0};
    return v[i];
  }
  __host__ __device__ static constexpr double a(int i, int j) {
    constexpr double v[13][14] = {
        {(1.0 / 18.0), 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {(1.0 / 48.0), (1.0 / 16.0), 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {(1.0 / 32.0), 0.0, (3.0 / 32.0), 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {(5.0 / 16.0), 0.0, (-75.0 / 64.0), (75.0 / 64.0), 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {(3.0 / 80.0), 0.0, 0.0, (3.0 / 16.0), (3.0 / 20.0), 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {(29443841.0 / 614563906.0), 0.0, 0.0, (77736538.0 / 692538347.0), (-28693883.0 / 1125000000.0), (23124283.0 / 1800000000.0), 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {(16016141.0 / 946692911.0), 0.0, 0.0, (61564180.0 / 158732637.0), (22789713.0 / 633445777.0), (545815736.0 / 2771057229.0), (-180193667.0 / 1043307555.0), 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {(39632708.0 / 573591083.0), 0.0, 0.0, (-433636366.0 / 683701615.0), (-421739975.0 / 2616292301.0), (100302831.0 / 723423059.0), (790204164.0 / 839813087.0), (800635310.0 / 3783071287.0), 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {(246121993.0 / 1340847787.0), 0.0, 0.0, (-37695042795.0 / 15268766246.0), (-309121744.0 / 1061227803.0), (-12992083.0 / 490766935.0), (6005943493.0 / 2108947869.0), (393006217.0 / 1396673457.0), (123872331.0 / 1001029789.0), 0.0, 0.0, 0.0, 0.0, 0.0},
        {(-1028468189.0 / 846180014.0), 0.0, 0.0, (8478235783.0 / 508512852.0), (1311729495.0 / 1432422823.0), (-10304129995.0 / 1701304382.0), (-48777925059.0 / 3047939560.0), (15336726248.0 / 1032824649.0), (-45442868181.0 / 3398467696.0), (3065993473.0 / 597172653.0), 0.0, 0.0, 0.0, 0.0},
        {(185892177.0 / 718116043.0), 0.0, 0.0, (-3185094517.0 / 667107341.0), (-477755414.0 / 1098053517.0), (-703635378.0 / 230739211.0), (5731566787.0 / 1027545527.0), (5232866602.0 / 850066563.0), (-4093664535.0 / 808688257.0), (3962137247.0 / 1805957418.0), (65686358.0 / 487910083.0), 0.0, 0.0, 0.0},
        {(403863854.0 / 491063109.0), 0.0, 0.0, (-5068492393.0 / 434740067.0), (-411421997.0 / 543043805.0), (652783627.0 / 914296604.0), (11173962825.0 / 925320556.0), (-13158990841.0 / 6184727034.0), (3936647629.0 / 1978049680.0), (-160528059.0 / 685178525.0), (248638103.0 / 1413531060.0), 0.0, 0.0, 0.0},
        {(14005451.0 / 335480064.0), 0.0, 0.0, 0.0, 0.0, (-59238493.0 / 1068277825.0), (181606767.0 / 758867731.0), (561292985.0 / 797845732.0), (-1041891430.0 / 1371343529.0), (760417239.0 / 1151165299.0), (118820643.0 / 751138087.0), (-528747749.0 / 2220607170.0), (1.0 / 4.0), 0.0},
    };
    return i == 0 ? 0.0 : v[i - 1][j];
  }
  __host__ __device__ static constexpr double b(int j) {
    constexpr double v[14] = {(14005451.0 / 335480064.0), 0.0, 0.0, 0.0, 0.0, (-59238493.0 / 1068277825.0), (181606767.0 / 758867731.0), (561292985.0 / 797845732.0), (-1041891430.0 / 1371343529.0), (760417239.0 / 1151165299.0), (118820643.0 / 751138087.0), (-528747749.0 / 2220607170.0), (1.0 / 4.0), 0.0};
    return v[j];
  }
  __host__ __device__ static constexpr double e(int j) {
    constexpr double v[14] = {((14005451.0 / 335480064.0) - (13451932.0 / 455176623.0)), 0.0, 0.0, 0.0, 0.0, ((-59238493.0 / 1068277825.0) - (-808719846.0 / 976000145.0)), ((181606767.0 / 758867731.0) - (1757004468.0 / 5645159321.0)), ((561292985.0 / 797845732.0) - (656045339.0 / 265891186.0)), ((-1041891430.0 / 1371343529.0) - (-3867574721.0 / 1518517206.0)), ((760417239.0 / 1151165299.0) - (465885868.0 / 322736535.0)), ((118820643.0 / 751138087.0) - (53011238.0 / 667516719.0)), ((-528747749.0 / 2220607170.0) - (2.0 / 45.0)), (1.0 / 4.0), 0.0};
    return v[j];
  }
  __host__ __device__ static constexpr double p(int j, int m) {
    constexpr double v[14][6] = {
        {-6.34483493928604, 22.139650499809406, -30.061056828966645, 19.999006933368396, -6.6910181737837595, 1.0},
        {0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
        {-39.61079198522025, 116.44221495503422, -121.49996277313346, 52.227353279294555, -7.6142658045872675, 0.0},
        {20.376121380879145, -67.14513188259572, 83.17210046398478, -46.89191641810936, 10.728139263042886, 0.0},
        {7.334709882679536, -16.56722435274965, 9.572450755599366, -0.18908932250105956, 0.5526637063753649, 0.0},
        {32.88017743524592, -89.9916014847245, 87.84060576772056, -35.70759759462221, 4.218656262566515, 0.0},
        {-10.158899052642676, 22.623748964853284, -17.415210777076297, 6.273644808324035, -0.6627209125361597, 0.0},
        {-12.540126809878256, 32.23623401673554, -28.590328951479098, 10.316088127245076, -1.2636789001135462, 0.0},
        {29.555300148451604, -82.10203154883598, 81.66309505843414, -34.76507698666118, 5.410603789859042, 0.0},
        {-41.79234864243906, 116.26621857911195, -114.93752913770093, 47.745797107822554, -7.032137906794574, 0.0},
        {20.300692582210083, -53.90207774663854, 50.255836422617605, -19.008209934160803, 2.3537586759714983, 0.0},
    };
    return v[j][m];
  }
};

// ---------------------------------------------------------------------------
// Precision helpers.
// ---------------------------------------------------------------------------
template <class T>
struct Math;
template <>
struct Math<float> {
  __device__ static __forceinline__ float sqrt_(float x) { return sqrtf(x); }
  __device__ static __forceinline__ float abs_(float x) { return fabsf(x); }
  __device__ static __forceinline__ float log2_(float x) { return log2f(x); }
  __device__ static __forceinline__ float exp2_(float x) { return exp2f(x); }
  __device__ static __forceinline__ float tanh_(float x) { return tanhf(x); }
};
template <>
struct Math<double> {
  __device__ static __forceinline__ double sqrt_(double x) { return sqrt(x); }
  __device__ static __forceinline__ double abs_(double x) { return fabs(x); }
  __device__ static __forceinline__ double log2_(double x) { return log2(x); }
  __device__ static __forceinline__ double exp2_(double x) { return exp2(x); }
  __device__ static __forceinline__ double tanh_(double x) { return tanh(x); }
};

__device__ __forceinline__ bool is_nan_(float x) { return isnan(x); }
__device__ __forceinline__ bool is_nan_(double x) { return isnan(x); }

// Order-preserving integer key of a double: key(a) < key(b) <=> a < b for
// non-NaN values (with -0 one below +0).  Comparisons on keys run on the
// integer pipes, which matters on GB300 where FP64 issue is ~1/64 of FP32.
__host__ __device__ __forceinline__ long long order_key(double x) {
#ifdef __CUDA_ARCH__
  long long b = __double_as_longlong(x);
#else
  long long b;
  memcpy(&b, &x, sizeof b);
#endif
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
__host__ __device__ __forceinline__ double from_order_key(long long k) {
  long long b = k >= 0 ? k : (k ^ 0x7fffffffffffffffLL);
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// nextafter(x, +inf) for finite x.
__device__ __forceinline__ double next_up(double x) {
  long long k = order_key(x) + 1;
  if (k == 0) k = 1;  // from -0 the next value up is +denorm_min
  return from_order_key(k);
}

// nextafter(x, -inf) for non-NaN x (+inf gives the largest finite double).
__device__ __forceinline__ double next_down(double x) {
  long long k = order_key(x) - 1;
  if (k == -1) k = -2;  // from +0 the next value down is -denorm_min
  return from_order_key(k);
}

// The ConstantStepSize grid fraction RN(s / n) (constant.py:84-86) for
// integers 0 < s <= n < 2^31, from inv = RN(1 / n) formed once per
// trajectory: q = RN(s inv) lies within one ulp of s / n, the remainder
// s - q n is exact under an FMA, and RN(q + r inv) is then the correctly
// rounded quotient (Markstein's theorem on the final correction step of
// Newton-Raphson division).  Three dependent FP64 operations instead of a
// division, whose dependent chain GB300's narrow FP64 pipe makes the longest
// part of a constant step.
__device__ __forceinline__ double grid_fraction(int s, int n, double inv) {
  const double sd = double(s);
  const double q = __dmul_rn(sd, inv);
  const double r = fma(-q, double(n), sd);
  return fma(r, inv, q);
}

// The grid time t0 + (t1 - t0) RN(s / n) rounded as the reference rounds it:
// a multiply, then an add, never contracted into an FMA (the FP32-state
// kernels are compiled with contraction on).
__device__ __forceinline__ double grid_time(double t0s, double t1s, int s, int n, double inv) {
  return __dadd_rn(t0s, __dmul_rn(t1s - t0s, grid_fraction(s, n, inv)));
}

// t1 minus 100 ULP (_integrate.py:319-322): 100 applications of
// nextafter(., -inf), the threshold above which tnext snaps to t1.
__device__ __forceinline__ double t1_clip_floor(double t1) {
  long long k = order_key(t1);
  long long k2 = k - 100;
  if (k >= 0 && k2 < 0) k2 -= 1;  // the key space holds both +0 and -0
  return from_order_key(k2);
}

struct SolveParams;

// ---------------------------------------------------------------------------
// Registered analytic vector fields.  All are autonomous, so stage times are
// never formed (runge_kutta.py:1023 computes them only to pass to vf).  A
// field may carry a diagonal diffusion (SDE = true, sigma()).
// ---------------------------------------------------------------------------
template <class T>
struct LotkaVolterra {
  static constexpr int D = 2, NARGS = 4;
  static constexpr bool SDE = false;
  static constexpr bool TAPE = false;  // no gradient tape (forward only)
  __device__ static __forceinline__ void vf(const SolveParams &, const T *a, const T *y, T *o) {
    o[0] = a[0] * y[0] - a[1] * y[0] * y[1];
    o[1] = -a[2] * y[1] + a[3] * y[0] * y[1];
  }
  // gy += (df/dy)^T g, ga += (df/da)^T g
  __device__ static __forceinline__ void vjp(const T *a, const T *y, const T *g, T *gy, T *ga) {
    gy[0] += g[0] * (a[0] - a[1] * y[1]) + g[1] * (a[3] * y[1]);
    gy[1] += g[0] * (-a[1] * y[0]) + g[1] * (-a[2] + a[3] * y[0]);
    ga[0] += g[0] * y[0];
    ga[1] += -g[0] * y[0] * y[1];
    ga[2] += -g[1] * y[1];
    ga[3] += g[1] * y[0] * y[1];
  }
};

template <class T>
struct VanDerPol {
  static constexpr int D = 2, NARGS = 1;
  static constexpr bool SDE = false;
  static constexpr bool TAPE = false;  // no gradient tape (forward only)
  __device__ static __forceinline__ void vf(const SolveParams &, const T *a, const T *y, T *o) {
    o[0] = y[1];
    o[1] = a[0] * (T(1) - y[0] * y[0]) * y[1] - y[0];
  }
  __device__ static __forceinline__ void vjp(const T *a, const T *y, const T *g, T *gy, T *ga) {
    gy[0] += g[1] * (T(-2) * a[0] * y[0] * y[1] - T(1));
    gy[1] += g[0] + g[1] * a[0] * (T(1) - y[0] * y[0]);
    ga[0] += g[1] * (T(1) - y[0] * y[0]) * y[1];
  }
};

template <class T, int D_>
struct OrnsteinUhlenbeck {
  static constexpr int D = D_, NARGS = 3;
  static constexpr bool SDE = false;
  static constexpr bool TAPE = false;  // no gradient tape (forward only)
  __device__ static __forceinline__ void vf(const SolveParams &, const T *a, const T *y, T *o) {
#pragma unroll
    for (int i = 0; i < D; i++) o[i] = a[0] * (a[1] - y[i]);
  }
  __device__ static __forceinline__ void vjp(const T *a, const T *y, const T *g, T *gy, T *ga) {
#pragma unroll
    for (int i = 0; i < D; i++) {
      gy[i] += -a[0] * g[i];
      ga[0] += g[i] * (a[1] - y[i]);
      ga[1] += g[i] * a[0];
    }
  }
};

// Ornstein-Uhlenbeck SDE: the drift above with the diagonal diffusion sigma of
// a ControlTerm driven by the virtual Brownian tree (dy = theta (mu - y) dt +
// sigma dW, _term.py:271-555 with a diagonal operator).  Brownian values come
// in pairs of components, so D is even.  LEVY_ selects the tree with
// space-time Levy area (levy_area=SpaceTimeLevyArea), which ShARK needs.
template <class T, int D_, bool LEVY_ = false>
struct OrnsteinUhlenbeckSDE : OrnsteinUhlenbeck<T, D_> {
  static_assert(D_ % 2 == 0, "the Brownian tree draws components in pairs");
  static constexpr bool SDE = true;
  static constexpr bool LEVY = LEVY_;
  __device__ static __forceinline__ void sigma(const SolveParams &, const T *a, const T *,
                                               T *s) {
#pragma unroll
    for (int i = 0; i < D_; i++) s[i] = a[2];
  }
  // VJP of y -> sigma(y) * dw (elementwise) with cotangent g: sigma is the
  // constant a[2], so only ga[2] receives sum_i g_i dw_i.
  __device__ static __forceinline__ void sigma_vjp(const T *, const T *, const T *dw,
                                                   const T *g, T *, T *ga) {
#pragma unroll
    for (int i = 0; i < D_; i++) ga[2] += g[i] * dw[i];
  }
};

// Whether a field's Brownian tree carries the space-time Levy area.
template <class F, class = void>
struct FieldLevy {
  static constexpr bool value = false;
};
template <class F>
struct FieldLevy<F, decltype(void(F::LEVY))> {
  static constexpr bool value = F::LEVY;
};

// ---------------------------------------------------------------------------
// Kernel parameters shared by every analytic-field launch.
// ---------------------------------------------------------------------------
struct SolveParams {
  int64_t batch;
  const double *t0, *t1, *dt0;
  int64_t time_stride;
  const void *y0;
  const void *args;
  int64_t args_stride;
  const void *params;
  const double *save_ts;
  void *ys_out;
  double *ts_out;
  int32_t *result_out;
  int32_t *stats_out;
  // controller / problem constants
  int controller;
  double rtol, atol, safety, factormin, factormax, dtmin, dtmax;
  int has_dtmin, has_dtmax, force_dtmin;
  double c1, c2, c3;  // PID exponents (i+p+d)/k, -(p+2d)/k, d/k
  // FP32 copies of the controller constants for the FP32-state kernels (the
  // FP64 pipe of GB300 issues at ~1/64 of the FP32 rate: no per-step
  // conversions)
  float rtol_f, atol_f, safety_f, factormin_f, factormax_f, c1_f, c2_f, c3_f;
  int n_ts, save_t0, save_t1, n_save, max_steps;
  int saves_prefilled;        // the unused save slots were filled before the launch
  unsigned long long *queue;  // work-stealing counter (fused kernel)
  const int32_t *order;       // optional work order: queue slot -> trajectory
  // MLP fields and SDEs
  const float *mlp;           // flat FP32 parameters (W0, b0, W1, b1, W2, b2, Ws, bs)
  const uint2 *w0f, *w2f;     // width 256: W0 and W2 as BF16 mma B fragments (workspace)
  uint64_t seed;              // Brownian generator seed
  double vbt_t0, vbt_len, vbt_tol_unit;
  double vbt_inv_len;         // 1 / vbt_len
  float vbt_sqrt_len;         // sqrt(vbt_len) as FP32
  // Recursive-checkpoint tape (forward pass of a differentiated solve)
  double *tape_t;             // [batch, max_steps + 1] accepted-step time grid
  float *tape_y;              // [batch, checkpoints, dim] state checkpoints
  int32_t *tape_n;            // [batch] accepted steps
  int32_t *tape_stride;       // [batch] accepted steps between checkpoints
  int checkpoints;
  // SaveAt(steps=n) and SaveAt(dense=True) (the extended-output kernels)
  int save_steps;             // n > 0: save (tnext, y1) of every n-th accepted step
  double *dense_ts;           // [batch, max_steps + 1] step times (direction-flipped)
  void *dense_info;           // [batch, max_steps, (2 + stages) dim]: y0, y1, k_j
  int32_t *dense_n;           // [batch] accepted steps + 1
  // ClipStepSizeController(step_ts, jump_ts) around the PID controller (the
  // extended-output kernels): caller-time times sorted increasing
  const double *step_ts, *jump_ts;
  int n_step_ts, n_jump_ts;
  // Event (the extended-output kernels): conditions, root finder, output
  int n_event, event_root;
  int ev_kind[GBDX_MAX_EVENTS], ev_dir[GBDX_MAX_EVENTS];
  double newton_rtol, newton_atol;
  double ev_coef[6 * GBDX_MAX_EVENTS];
  int32_t *event_index;       // [batch] condition that ended the solve, -1 none
  // Resuming (gbdx_fwd_extras): [batch, GBDX_STATE_HEAD + dim] FP64 records
  const double *state_in;
  double *state_out;
  // Bounds-checked builds: the first out-of-range index (site << 56 | index)
  // and the sink that takes its access (null in release builds)
  unsigned long long *bounds;
  void *bounds_sink;
};

// GBDX_AT(P, base, off, width, extent, site): base + off, where the access
// covers elements [off, off + width) of a buffer of `extent` elements.  In a
// bounds-checked build (-DGBDX_BOUNDS) an access outside [0, extent) records
// (site, off) in P.bounds -- the first of the launch -- and goes to
// P.bounds_sink instead (GBDX_BOUNDS_BYTES - 256 bytes); the release build
// compiles to the plain pointer arithmetic.
#ifdef GBDX_BOUNDS
template <class T>
__device__ __forceinline__ T *bounds_at(unsigned long long *rec, void *sink, T *base,
                                        int64_t off, int64_t width, int64_t extent, int site) {
  if (off >= 0 && off + width <= extent) return base + off;
  atomicCAS(rec, 0ull,
            (static_cast<unsigned long long>(site) << 56) |
                (static_cast<unsigned long long>(off) & 0x00ffffffffffffffull));
  return reinterpret_cast<T *>(sink);
}
#define GBDX_AT(P, base, off, width, extent, site)                                     \
  ::gbdx::bounds_at((P).bounds, (P).bounds_sink, (base), int64_t(off), int64_t(width), \
                    int64_t(extent), (site))
#else
#define GBDX_AT(P, base, off, width, extent, site) ((base) + (off))
#endif

// BacksolveAdjoint backward arguments.
struct BsParams {
  const float *ys;       // [batch, n_save, D] the forward's saved states
  const float *grad_ys;  // [batch, n_save, D]
  float *grad_y0;        // [batch, D]
  float *psum, *pcomp;   // [n_cta, NP] Kahan partial gradients
  float *rec;            // [n_cta, S, M, REC] stage records
  float *ath;            // [n_cta, M, 2, NP] per-row a_theta (tracked norm only)
  const uint2 *w0f, *w0v, *w2f, *w2v;  // B fragments (width 256)
  int track;             // the error norm runs over a_theta
  float n_norm;          // number of components in the error norm
};

// Arguments of the analytic-field backward kernels (device pointers in the
// problem's dtype).
struct AdjParams {
  const void *grad_ys;  // [batch, n_save, D]
  const void *ys;       // backsolve: the forward's saved states [batch, n_save, D]
  void *grad_y0;        // [batch, D]
  void *grad_args;      // [batch, n_args] per trajectory
  int track_args;       // backsolve: the error norm covers a_args (rms_norm)
};

// Backward (RecursiveCheckpointAdjoint) arguments.
struct BwdParams {
  const float *grad_ys;   // [batch, n_save, D]
  float *grad_y0;         // [batch, D]
  float *part_sum;        // [n_cta, n_params] per-CTA partial gradients
  float *part_comp;       // [n_cta, n_params] Kahan compensation
  float *scratch;         // [batch, seg_max, D] segment recompute states
  int seg_max;
  int n_params;
};

}  // namespace gbdx

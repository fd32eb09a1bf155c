/*
 * gbdx_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * An FP64 CPU restatement of Diffrax's batched `diffeqsolve` hot path, used as
 * the parity oracle for the CUDA kernels and as the timed CPU baseline.  It is
 * never linked into, loaded by, or called from the product library; only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it.
 *
 * Each block below names the reference file:line it restates (paths are
 * relative to the Diffrax source tree, v0.7.2).
 *
 *   solve loop ............ diffrax/_integrate.py:302-885, 1036-1305
 *   explicit RK step ...... diffrax/_solver/runge_kutta.py:446-1203
 *   tableaus .............. diffrax/_solver/{tsit5,dopri5,dopri8,heun,euler}.py
 *   interpolants .......... diffrax/_solver/tsit5.py:103-156, dopri8.py:192-303,
 *                           diffrax/_local_interpolation.py:29-139
 *   PID controller ........ diffrax/_step_size_controller/pid.py:316-567
 *   constant step size .... diffrax/_step_size_controller/constant.py:20-104
 *   clip controller ....... diffrax/_step_size_controller/clip.py:36-427
 *                           (step_ts, jump_ts; no store_rejected_steps)
 *   events ................ diffrax/_event.py:13-175 (registered conditions),
 *                           diffrax/_integrate.py:542-633 (detection),
 *                           686-821 (root find and unsave), 847-877, with
 *                           optimistix.Newton (cauchy termination) restated
 *   terms ................. diffrax/_term.py:174-226, 271-555, 666-764
 *   virtual Brownian tree . diffrax/_brownian/tree.py:94-126, 245-354, 366-448,
 *                           562-621, 626-773 (BrownianIncrement and
 *                           SpaceTimeLevyArea branches)
 *   additive-noise SRKs ... diffrax/_solver/{shark,sra1,sea}.py:10-35 with
 *                           the additive-noise step of diffrax/_solver/srk.py:
 *                           335-671
 *   gradients ............. diffrax/_adjoint.py:179-312 (discretise-then-
 *                           optimise: exact VJP of the accepted-step map with
 *                           the controller under stop_gradient, pid.py:374,
 *                           499-501, 529-530), diffrax/_adjoint.py:538-734 and
 *                           diffrax/_term.py:767-910 (backsolve).
 *
 * Built with -ffp-contract=off so that x86-64 and aarch64 give identical bits.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { ORC_EULER = 0, ORC_HEUN = 1, ORC_DOPRI5 = 2, ORC_TSIT5 = 3, ORC_DOPRI8 = 4,
       ORC_SHARK = 5, ORC_SRA1 = 6, ORC_SEA = 7 };
/* the additive-noise stochastic Runge-Kutta methods (srk.py) */
#define ORC_IS_SRK(s) ((s) == ORC_SHARK || (s) == ORC_SRA1 || (s) == ORC_SEA)
#define ORC_MAX_S 14 /* most stages of a tableau (Dopri8) */
enum { ORC_CONSTANT = 0, ORC_PID = 1 };
enum {
  ORC_LOTKA_VOLTERRA = 0,
  ORC_VAN_DER_POL = 1,
  ORC_ORNSTEIN_UHLENBECK = 2,
  ORC_MLP = 3,
  ORC_LINEAR = 4,   /* y' = A y, A a dim x dim matrix passed as params */
  ORC_CALLBACK = 5  /* arbitrary host callback, forward only */
};
enum { ORC_DIFF_NONE = 0, ORC_DIFF_OU = 1, ORC_DIFF_TANH_DIAG = 2 };
enum { ORC_NORM_RMS = 0, ORC_NORM_ADJOINT_SEMI = 1 };
/* Registered event conditions: a linear form w.y + wt t + c of the state and
 * the loop's time (real-valued, or its sign as a boolean), and
 * steady_state_event (boolean, _event.py:120-175). */
enum { ORC_EV_LINEAR = 0, ORC_EV_LINEAR_BOOL = 1, ORC_EV_STEADY = 2 };
enum { ORC_EV_EITHER = 0, ORC_EV_UP = 1, ORC_EV_DOWN = 2 };
#define ORC_MAX_EVENTS 4

/* RESULTS codes (diffrax/_solution.py:13-31): successful must be 0. */
enum {
  ORC_SUCCESSFUL = 0,
  ORC_MAX_STEPS_REACHED = 1,
  ORC_DT_MIN_REACHED = 2,
  ORC_EVENT_OCCURRED = 3,
  ORC_MAX_STEPS_REJECTED = 4,
  ORC_INTERNAL_ERROR = 5,
  ORC_EVENT_ROOT_MAX_STEPS = 6 /* the event's root find did not converge */
};

typedef void (*orc_vf_cb)(double t, const double *y, double *out, int dim,
                          void *ctx);

/* Mirrors the problem descriptor of the product ABI (include/gbdx.h). */
typedef struct {
  int32_t solver, controller, field, dim;
  double rtol, atol, pcoeff, icoeff, dcoeff, safety, factormin, factormax;
  double dtmin, dtmax; /* NaN = None */
  int32_t force_dtmin;
  double error_order; /* 0 = solver default */
  int32_t n_ts, save_t0, save_t1, max_steps;
  int32_t n_args;
  int32_t mlp_depth;      /* number of linear layers */
  int32_t mlp_widths[9];  /* widths[0] = in, widths[depth] = out */
  int32_t diffusion;      /* ORC_DIFF_* */
  double vbt_t0, vbt_t1, vbt_tol;
  uint64_t seed;
  int32_t norm;           /* used by the backsolve adjoint only */
  int32_t save_steps;     /* SaveAt(steps=n): every n-th accepted step; 0 = off */
  int32_t save_dense;     /* SaveAt(dense=True) */
  /* ClipStepSizeController(step_ts, jump_ts) around the PID controller: the
   * times follow the n_ts SaveAt times in the solve's `ts` array, each group
   * sorted increasing in the caller's time */
  int32_t n_step_ts, n_jump_ts;
  /* Event(cond_fn=[...], root_finder, direction): n_event conditions of kind
   * ev_kind (ORC_EV_*) and direction ev_dir (ORC_EV_EITHER/UP/DOWN); linear:
   * ev_coef[6 i + n] = w_n (n < min(dim, 4)), [6 i + 4] = wt, [6 i + 5] = c;
   * steady state: [6 i] = rtol, [6 i + 1] = atol.  event_root = 1 finds the
   * event time by Newton's method with newton_rtol / newton_atol. */
  int32_t n_event, event_root;
  int32_t ev_kind[ORC_MAX_EVENTS], ev_dir[ORC_MAX_EVENTS];
  /* the tree's Levy area: 0 = BrownianIncrement, 1 = SpaceTimeLevyArea */
  int32_t levy_area;
  double newton_rtol, newton_atol;
  double ev_coef[6 * ORC_MAX_EVENTS];
} orc_desc;

/* ------------------------------------------------------------------------ */
/* Butcher tableaus.  Coefficients are the published method constants as the */
/* reference writes them (tsit5.py:18-100, dopri5.py:11-33, heun.py:12-17); */
/* the error rows are evaluated as the same FP64 differences.                */
/* ------------------------------------------------------------------------ */
typedef struct {
  int s;          /* stages */
  int fsal, ssal; /* runge_kutta.py:143-165 */
  double a[ORC_MAX_S][ORC_MAX_S]; /* a[i][j], j < i */
  double b[ORC_MAX_S], e[ORC_MAX_S], c[ORC_MAX_S];
  int order;      /* ODE order; error_order for ODEs (base.py:97-120) */
  double strong_order;
  /* additive-noise SRK (srk.py AdditiveCoeffs): stage j adds
   * g (aw[j] W + ah[j] H), the solution g (bw W + bh H); has_err = 0 when the
   * tableau has no b_error */
  double aw[ORC_MAX_S], ah[ORC_MAX_S], bw, bh;
  int has_err;
} Tableau;

static Tableau TSIT5, DOPRI5, DOPRI8, HEUN, EULER, SHARK, SRA1, SEA;
/* Dopri8 (dopri8.py:18-189): Prince and Dormand's 8(7) pair, 14 stages,
 * FSAL and SSAL; published method constants as exact rational quotients. */
static const double DOPRI8_A[13][ORC_MAX_S] = {
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
static const double DOPRI8_B[ORC_MAX_S] = {(14005451.0 / 335480064.0), 0.0, 0.0, 0.0, 0.0, (-59238493.0 / 1068277825.0), (181606767.0 / 758867731.0), (561292985.0 / 797845732.0), (-1041891430.0 / 1371343529.0), (760417239.0 / 1151165299.0), (118820643.0 / 751138087.0), (-528747749.0 / 2220607170.0), (1.0 / 4.0), 0.0};
static const double DOPRI8_E[ORC_MAX_S] = {((14005451.0 / 335480064.0) - (13451932.0 / 455176623.0)), 0.0, 0.0, 0.0, 0.0, ((-59238493.0 / 1068277825.0) - (-808719846.0 / 976000145.0)), ((181606767.0 / 758867731.0) - (1757004468.0 / 5645159321.0)), ((561292985.0 / 797845732.0) - (656045339.0 / 265891186.0)), ((-1041891430.0 / 1371343529.0) - (-3867574721.0 / 1518517206.0)), ((760417239.0 / 1151165299.0) - (465885868.0 / 322736535.0)), ((118820643.0 / 751138087.0) - (53011238.0 / 667516719.0)), ((-528747749.0 / 2220607170.0) - (2.0 / 45.0)), (1.0 / 4.0), 0.0};
static const double DOPRI8_C[ORC_MAX_S] = {0.0, (1.0 / 18.0), (1.0 / 12.0), (1.0 / 8.0), (5.0 / 16.0), (3.0 / 8.0), (59.0 / 400.0), (93.0 / 200.0), (5490023248.0 / 9719169821.0), (13.0 / 20.0), (1201146811.0 / 1299019798.0), 1.0, 1.0, 1.0};
/* Bogacki--Shampine dense output of Dopri8 (dopri8.py:192-303):
 * y(theta) = y0 + sum_j theta * P_j(theta) k_j with P_j the degree-5
 * polynomial of row j (highest power first). */
static const double DOPRI8_P[ORC_MAX_S][6] = {
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


static void init_tableaus(void) {
  static int done = 0;
  if (done) return;
  memset(&TSIT5, 0, sizeof TSIT5);
  TSIT5.s = 7; TSIT5.fsal = 1; TSIT5.ssal = 1; TSIT5.order = 5;
  TSIT5.strong_order = 0.0;
  TSIT5.c[1] = 161.0 / 1000; TSIT5.c[2] = 327.0 / 1000; TSIT5.c[3] = 9.0 / 10;
  TSIT5.c[4] = 0.9800255409045096857298102862870245954942137979563024768854764293221195950761080302604;
  TSIT5.c[5] = 1.0; TSIT5.c[6] = 1.0;
  TSIT5.a[1][0] = 161.0 / 1000;
  TSIT5.a[2][0] = -0.8480655492356988544426874250230774675121177393430391537369234245294192976164141156943e-2;
  TSIT5.a[2][1] = 0.3354806554923569885444268742502307746751211773934303915373692342452941929761641411569;
  TSIT5.a[3][0] = 2.897153057105493432130432594192938764924887287701866490314866693455023795137503079289;
  TSIT5.a[3][1] = -6.359448489975074843148159912383825625952700647415626703305928850207288721235210244366;
  TSIT5.a[3][2] = 4.362295432869581411017727318190886861027813359713760212991062156752264926097707165077;
  TSIT5.a[4][0] = 5.325864828439256604428877920840511317836476253097040101202360397727981648835607691791;
  TSIT5.a[4][1] = -11.74888356406282787774717033978577296188744178259862899288666928009020615663593781589;
  TSIT5.a[4][2] = 7.495539342889836208304604784564358155658679161518186721010132816213648793440552049753;
  TSIT5.a[4][3] = -0.9249506636175524925650207933207191611349983406029535244034750452930469056411389539635e-1;
  TSIT5.a[5][0] = 5.861455442946420028659251486982647890394337666164814434818157239052507339770711679748;
  TSIT5.a[5][1] = -12.92096931784710929170611868178335939541780751955743459166312250439928519268343184452;
  TSIT5.a[5][2] = 8.159367898576158643180400794539253485181918321135053305748355423955009222648673734986;
  TSIT5.a[5][3] = -0.7158497328140099722453054252582973869127213147363544882721139659546372402303777878835e-1;
  TSIT5.a[5][4] = -0.2826905039406838290900305721271224146717633626879770007617876201276764571291579142206e-1;
  {
    const double bs[6] = {
        0.9646076681806522951816731316512876333711995238157997181903319145764851595234062815396e-1,
        1.0 / 100,
        0.4798896504144995747752495322905965199130404621990332488332634944254542060153074523509,
        1.379008574103741893192274821856872770756462643091360525934940067397245698027561293331,
        -3.290069515436080679901047585711363850115683290894936158531296799594813811049925401677,
        2.324710524099773982415355918398765796109060233222962411944060046314465391054716027841};
    for (int j = 0; j < 6; j++) { TSIT5.a[6][j] = bs[j]; TSIT5.b[j] = bs[j]; }
    TSIT5.b[6] = 0.0;
    TSIT5.e[0] = bs[0] - 0.9468075576583945807478876255758922856117527357724631226139574065785592789071067303271e-1;
    TSIT5.e[1] = bs[1] - 0.9183565540343253096776363936645313759813746240984095238905939532922955247253608687270e-2;
    TSIT5.e[2] = bs[2] - 0.4877705284247615707855642599631228241516691959761363774365216240304071651579571959813;
    TSIT5.e[3] = bs[3] - 1.234297566930478985655109673884237654035539930748192848315425833500484878378061439761;
    TSIT5.e[4] = bs[4] + 2.707712349983525454881109975059321670689605166938197378763992255714444407154902012702;
    TSIT5.e[5] = bs[5] - 1.866628418170587035753719399566211498666255505244122593996591602841258328965767580089;
    TSIT5.e[6] = -1.0 / 66;
  }

  memset(&DOPRI5, 0, sizeof DOPRI5);
  DOPRI5.s = 7; DOPRI5.fsal = 1; DOPRI5.ssal = 1; DOPRI5.order = 5;
  DOPRI5.c[1] = 1.0 / 5; DOPRI5.c[2] = 3.0 / 10; DOPRI5.c[3] = 4.0 / 5;
  DOPRI5.c[4] = 8.0 / 9; DOPRI5.c[5] = 1.0; DOPRI5.c[6] = 1.0;
  DOPRI5.a[1][0] = 1.0 / 5;
  DOPRI5.a[2][0] = 3.0 / 40; DOPRI5.a[2][1] = 9.0 / 40;
  DOPRI5.a[3][0] = 44.0 / 45; DOPRI5.a[3][1] = -56.0 / 15; DOPRI5.a[3][2] = 32.0 / 9;
  DOPRI5.a[4][0] = 19372.0 / 6561; DOPRI5.a[4][1] = -25360.0 / 2187;
  DOPRI5.a[4][2] = 64448.0 / 6561; DOPRI5.a[4][3] = -212.0 / 729;
  DOPRI5.a[5][0] = 9017.0 / 3168; DOPRI5.a[5][1] = -355.0 / 33;
  DOPRI5.a[5][2] = 46732.0 / 5247; DOPRI5.a[5][3] = 49.0 / 176;
  DOPRI5.a[5][4] = -5103.0 / 18656;
  DOPRI5.a[6][0] = 35.0 / 384; DOPRI5.a[6][1] = 0.0; DOPRI5.a[6][2] = 500.0 / 1113;
  DOPRI5.a[6][3] = 125.0 / 192; DOPRI5.a[6][4] = -2187.0 / 6784; DOPRI5.a[6][5] = 11.0 / 84;
  for (int j = 0; j < 6; j++) DOPRI5.b[j] = DOPRI5.a[6][j];
  DOPRI5.b[6] = 0.0;
  DOPRI5.e[0] = 35.0 / 384 - 1951.0 / 21600;
  DOPRI5.e[1] = 0.0;
  DOPRI5.e[2] = 500.0 / 1113 - 22642.0 / 50085;
  DOPRI5.e[3] = 125.0 / 192 - 451.0 / 720;
  DOPRI5.e[4] = -2187.0 / 6784 - -12231.0 / 42400;
  DOPRI5.e[5] = 11.0 / 84 - 649.0 / 6300;
  DOPRI5.e[6] = -1.0 / 60.0;

  memset(&DOPRI8, 0, sizeof DOPRI8);
  DOPRI8.s = 14; DOPRI8.fsal = 1; DOPRI8.ssal = 1; DOPRI8.order = 8;
  for (int i = 1; i < 14; i++)
    for (int j = 0; j < i; j++) DOPRI8.a[i][j] = DOPRI8_A[i - 1][j];
  for (int j = 0; j < 14; j++) {
    DOPRI8.b[j] = DOPRI8_B[j];
    DOPRI8.e[j] = DOPRI8_E[j];
    DOPRI8.c[j] = DOPRI8_C[j];
  }

  memset(&HEUN, 0, sizeof HEUN);
  HEUN.s = 2; HEUN.fsal = 0; HEUN.ssal = 0; HEUN.order = 2; HEUN.strong_order = 0.5;
  HEUN.c[1] = 1.0; HEUN.a[1][0] = 1.0;
  HEUN.b[0] = 0.5; HEUN.b[1] = 0.5; HEUN.e[0] = 0.5; HEUN.e[1] = -0.5;

  memset(&EULER, 0, sizeof EULER);
  EULER.s = 1; EULER.order = 1; EULER.strong_order = 0.5; EULER.b[0] = 1.0;

  /* ShARK (shark.py:10-35) */
  memset(&SHARK, 0, sizeof SHARK);
  SHARK.s = 2; SHARK.order = 2; SHARK.strong_order = 1.5; SHARK.has_err = 1;
  SHARK.c[1] = 5.0 / 6.0; SHARK.a[1][0] = 5.0 / 6.0;
  SHARK.b[0] = 0.4; SHARK.b[1] = 0.6; SHARK.e[0] = -0.6; SHARK.e[1] = 0.6;
  SHARK.aw[0] = 0.0; SHARK.aw[1] = 5.0 / 6.0; SHARK.ah[0] = 1.0; SHARK.ah[1] = 1.0;
  SHARK.bw = 1.0; SHARK.bh = 0.0;

  /* SRA1 (sra1.py:10-34, Roessler 2010) */
  memset(&SRA1, 0, sizeof SRA1);
  SRA1.s = 2; SRA1.order = 2; SRA1.strong_order = 1.5; SRA1.has_err = 1;
  SRA1.c[1] = 3.0 / 4.0; SRA1.a[1][0] = 3.0 / 4.0;
  SRA1.b[0] = 1.0 / 3.0; SRA1.b[1] = 2.0 / 3.0; SRA1.e[0] = -2.0 / 3.0; SRA1.e[1] = 2.0 / 3.0;
  SRA1.aw[0] = 0.0; SRA1.aw[1] = 3.0 / 4.0; SRA1.ah[0] = 0.0; SRA1.ah[1] = 1.5;
  SRA1.bw = 1.0; SRA1.bh = 0.0;

  /* SEA, the shifted Euler method (sea.py:10-34): no error estimate */
  memset(&SEA, 0, sizeof SEA);
  SEA.s = 1; SEA.order = 1; SEA.strong_order = 1.0; SEA.has_err = 0;
  SEA.b[0] = 1.0; SEA.aw[0] = 0.5; SEA.ah[0] = 1.0; SEA.bw = 1.0; SEA.bh = 0.0;
  done = 1;
}

static const Tableau *tableau_of(int solver) {
  switch (solver) {
    case ORC_EULER: return &EULER;
    case ORC_HEUN: return &HEUN;
    case ORC_DOPRI5: return &DOPRI5;
    case ORC_DOPRI8: return &DOPRI8;
    case ORC_SHARK: return &SHARK;
    case ORC_SRA1: return &SRA1;
    case ORC_SEA: return &SEA;
    default: return &TSIT5;
  }
}

/* Dopri5 dense-output midpoint weights (dopri5.py:36-47). */
static const double DOPRI5_CMID[7] = {
    6025192743.0 / 30085553152.0 / 2, 0.0, 51252292925.0 / 65400821598.0 / 2,
    -2691868925.0 / 45128329728.0 / 2, 187940372067.0 / 1594534317056.0 / 2,
    -1776094331.0 / 19743644256.0 / 2, 11237099.0 / 235043384.0 / 2};

/* ------------------------------------------------------------------------ */
/* Counter-based normal generator (Philox4x32-10, Salmon et al. 2011) and the */
/* virtual Brownian tree that consumes it.  The kernels use the same integer  */
/* stream; only the uniform -> normal transform differs in precision.        */
/* ------------------------------------------------------------------------ */
static void philox4x32_10(uint32_t ctr[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * ctr[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * ctr[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ ctr[1] ^ k0, n2 = hi0 ^ ctr[3] ^ k1;
    ctr[0] = n0; ctr[1] = lo1; ctr[2] = n2; ctr[3] = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
}

enum { VBT_ROOT = 0, VBT_MID = 1, VBT_LEAF = 2 };

/* Four standard normals for (trajectory, tree node, draw kind, dims 4q..4q+3). */
static void normal4(uint64_t seed, uint32_t traj, uint32_t node, uint32_t kind,
                    uint32_t q, double z[4]) {
  uint32_t c[4] = {traj, node, (kind << 24) | q, 0x5EEDu};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  double u[4];
  for (int i = 0; i < 4; i++) u[i] = ((double)(c[i] >> 8) + 0.5) * (1.0 / 16777216.0);
  const double two_pi = 6.283185307179586476925286766559;
  double r0 = sqrt(-2.0 * log(u[0])), r1 = sqrt(-2.0 * log(u[2]));
  z[0] = r0 * cos(two_pi * u[1]); z[1] = r0 * sin(two_pi * u[1]);
  z[2] = r1 * cos(two_pi * u[3]); z[3] = r1 * sin(two_pi * u[3]);
}

static void normals(uint64_t seed, uint32_t traj, uint32_t node, uint32_t kind,
                    int dim, double *out) {
  for (int q = 0; q * 4 < dim; q++) {
    double z[4];
    normal4(seed, traj, node, kind, (uint32_t)q, z);
    for (int i = 0; i < 4 && q * 4 + i < dim; i++) out[q * 4 + i] = z[i];
  }
}

/* W(r) on the unit interval by binary bridge descent: tree.py:366-448 (loop),
 * 626-773 (BrownianIncrement arch, lines 752-768), 607-621 (final bridge). */
static void vbt_eval_unit(uint64_t seed, uint32_t traj, double tol_unit, double r,
                          int dim, double *w_r) {
  double ws[64], wu[64], wsu[64], z[64];
  int level = 0;
  double s = 0.0;
  uint32_t node = 1;
  normals(seed, traj, 0, VBT_ROOT, dim, z);
  for (int i = 0; i < dim; i++) { ws[i] = 0.0; wu[i] = z[i]; wsu[i] = z[i]; }
  while (ldexp(1.0, -level) > tol_unit) {
    double su = ldexp(1.0, -level);
    double st = su / 2;
    double t = s + st;
    double root_su = sqrt(su);
    normals(seed, traj, node, VBT_MID, dim, z);
    int right = r > t;
    for (int i = 0; i < dim; i++) {
      double mean = 0.5 * wsu[i];
      double term2 = (root_su / 2) * z[i];
      double w_st = mean + term2, w_tu = mean - term2;
      double w_t = ws[i] + w_st;
      if (right) { ws[i] = w_t; wsu[i] = w_tu; }
      else { wu[i] = w_t; wsu[i] = w_st; }
    }
    if (right) s = t;
    node = 2 * node + (uint32_t)right;
    level++;
  }
  double su = ldexp(1.0, -level);
  double sr = r - s; if (sr < 0) sr = 0;
  double ru = su - sr; if (ru < 0) ru = 0;
  normals(seed, traj, node, VBT_LEAF, dim, z);
  double bbs = sqrt(sr * ru / su);
  for (int i = 0; i < dim; i++) w_r[i] = (ws[i] + sr / su * wsu[i]) + bbs * z[i];
  (void)wu;
}

/* VirtualBrownianTree.evaluate(ta, tb) (tree.py:325-354): rescale to [0,1],
 * difference of two evaluations, multiply by sqrt(T). */
static void vbt_increment(const orc_desc *d, uint32_t traj, double ta, double tb,
                          double *dw) {
  double T = d->vbt_t1 - d->vbt_t0;
  double tol_unit = d->vbt_tol / T;
  double ra = (ta - d->vbt_t0) / T, rb = (tb - d->vbt_t0) / T;
  double wa[64], wb[64];
  vbt_eval_unit(d->seed, traj, tol_unit, ra, d->dim, wa);
  vbt_eval_unit(d->seed, traj, tol_unit, rb, d->dim, wb);
  double sq = sqrt(T);
  for (int i = 0; i < d->dim; i++) dw[i] = sq * (wb[i] - wa[i]);
}

/* The tree with space-time Levy area (levy_area = SpaceTimeLevyArea): the
 * descent carries W and bar H (bar H_{s,u} = (u - s) H_{s,u}) of each dyadic
 * interval.  Root: W_1 ~ N(0, 1), bar H_1 ~ N(0, 1/12) (tree.py:389-394);
 * midpoint rule tree.py:727-750 (Foster's thesis, Theorem 6.1.4 bridge);
 * final bridge to r tree.py:562-603.  Draws: VBT_ROOT / VBT_MID / VBT_LEAF
 * feed W (z1, x1), the _H kinds feed bar H (z2, x2). */
enum { VBT_ROOT_H = 3, VBT_MID_H = 4, VBT_LEAF_H = 5 };

static void vbt_levy_eval_unit(uint64_t seed, uint32_t traj, double tol_unit, double r,
                               int dim, double *w_r, double *bhh_r) {
  double ws[64], wsu[64], hs[64], hsu[64], z1[64], z2[64];
  int level = 0;
  double s = 0.0;
  uint32_t node = 1;
  normals(seed, traj, 0, VBT_ROOT, dim, z1);
  normals(seed, traj, 0, VBT_ROOT_H, dim, z2);
  for (int i = 0; i < dim; i++) {
    ws[i] = 0.0; wsu[i] = z1[i];
    hs[i] = 0.0; hsu[i] = z2[i] / sqrt(12.0);
  }
  while (ldexp(1.0, -level) > tol_unit) {
    double su = ldexp(1.0, -level);
    double st = su / 2;
    double t = s + st;
    double root_su = sqrt(su);
    normals(seed, traj, node, VBT_MID, dim, z1);
    normals(seed, traj, node, VBT_MID_H, dim, z2);
    int right = r > t;
    for (int i = 0; i < dim; i++) {
      double z = z1[i] * (root_su / 4);
      double n = z2[i] * sqrt(su / 12);
      double w_term1 = wsu[i] / 2;
      double w_term2 = (3 / (2 * su)) * hsu[i] + z;
      double w_st = w_term1 + w_term2, w_tu = w_term1 - w_term2;
      double h_term1 = hsu[i] / 8 - su / 4 * z;
      double h_term2 = (su / 4) * n;
      double h_st = h_term1 + h_term2, h_tu = h_term1 - h_term2;
      double w_t = ws[i] + w_st;
      double h_t = hs[i] + h_st + 0.5 * (t * ws[i] - s * w_t);
      if (right) { ws[i] = w_t; wsu[i] = w_tu; hs[i] = h_t; hsu[i] = h_tu; }
      else { wsu[i] = w_st; hsu[i] = h_st; }
    }
    if (right) s = t;
    node = 2 * node + (uint32_t)right;
    level++;
  }
  double su = ldexp(1.0, -level);
  double sr = r - s; if (sr < 0) sr = 0;
  double ru = su - sr; if (ru < 0) ru = 0;
  normals(seed, traj, node, VBT_LEAF, dim, z1);
  normals(seed, traj, node, VBT_LEAF_H, dim, z2);
  double sr3 = pow(sr, 3), ru3 = pow(ru, 3), su3 = pow(su, 3);
  double sr_ru_half = sqrt(sr * ru);
  double dd = sqrt(sr3 + ru3);
  double d_prime = 1 / (2 * su * dd);
  double a = d_prime * sr3 * sr_ru_half;
  double b = d_prime * ru3 * sr_ru_half;
  double c = sqrt(3 * sr3 * ru3) / (6 * dd);
  for (int i = 0; i < dim; i++) {
    double w_sr = sr / su * wsu[i] + 6 * sr * ru / su3 * hsu[i] + 2 * (a + b) / su * z1[i];
    w_r[i] = ws[i] + w_sr;
    double bhh_sr = sr3 / su3 * hsu[i] - a * z1[i] + c * z2[i];
    bhh_r[i] = hs[i] + bhh_sr + 0.5 * (r * ws[i] - s * w_r[i]);
  }
}

/* VirtualBrownianTree.evaluate(ta, tb, use_levy=True) (tree.py:325-354):
 * (W, H) of [ta, tb] from the two point values by Chen's relation
 * (_levy_diff, tree.py:94-126), then scaled by sqrt(T). */
static void vbt_levy_increment(const orc_desc *d, uint32_t traj, double ta, double tb,
                               double *dw, double *dh) {
  double T = d->vbt_t1 - d->vbt_t0;
  double tol_unit = d->vbt_tol / T;
  double ra = (ta - d->vbt_t0) / T, rb = (tb - d->vbt_t0) / T;
  double wa[64], wb[64], ha[64], hb[64];
  vbt_levy_eval_unit(d->seed, traj, tol_unit, ra, d->dim, wa, ha);
  vbt_levy_eval_unit(d->seed, traj, tol_unit, rb, d->dim, wb, hb);
  double su = rb - ra;
  double inv = fabs(su) < DBL_EPSILON ? 0.0 : 1 / su;
  double sq = sqrt(T);
  for (int i = 0; i < d->dim; i++) {
    double u_bb_s = rb * wa[i] - ra * wb[i];
    double bhh_su = hb[i] - ha[i] - 0.5 * u_bb_s;
    dw[i] = sq * (wb[i] - wa[i]);
    dh[i] = sq * (inv * bhh_su);
  }
}

/* The Brownian increment of the loop's step [tprev, tnext] (direction-
 * flipped time).  The WrapTerm (_term.py:742-745) evaluates the forward real
 * interval and multiplies the whole increment (W and H) by the direction. */
static void step_increment(const orc_desc *d, uint32_t traj, int dir, double tprev,
                           double tnext, double *dw, double *dh) {
  if (!d->levy_area) {
    vbt_increment(d, traj, dir * tprev, dir * tnext, dw);
    return;
  }
  if (dir > 0) {
    vbt_levy_increment(d, traj, tprev, tnext, dw, dh);
  } else {
    vbt_levy_increment(d, traj, -tnext, -tprev, dw, dh);
    for (int i = 0; i < d->dim; i++) { dw[i] = -dw[i]; dh[i] = -dh[i]; }
  }
}

/* ------------------------------------------------------------------------ */
/* Vector fields.                                                            */
/* ------------------------------------------------------------------------ */
typedef struct {
  const orc_desc *d;
  const double *args;   /* this trajectory's analytic args */
  const double *params; /* MLP / linear / diffusion parameters (flat) */
  orc_vf_cb cb;
  void *cb_ctx;
} Field;

/* Flat MLP layout: for each layer l, W_l [out x in] row-major then b_l [out];
 * then (diffusion ORC_DIFF_TANH_DIAG) W_sigma [dim x dim], b_sigma [dim]. */
static int64_t mlp_param_count(const orc_desc *d) {
  int64_t n = 0;
  for (int l = 0; l < d->mlp_depth; l++)
    n += (int64_t)d->mlp_widths[l] * d->mlp_widths[l + 1] + d->mlp_widths[l + 1];
  return n;
}

#define MAXW 512

/* eqx.nn.MLP semantics: tanh on hidden layers, identity output.  When acts is
 * non-NULL the hidden activations are stored for the VJP. */
static void mlp_forward(const orc_desc *d, const double *P, const double *x,
                        double *out, double *acts) {
  double buf0[MAXW], buf1[MAXW];
  const double *in = x;
  double *cur = buf0;
  const double *p = P;
  int aoff = 0;
  for (int l = 0; l < d->mlp_depth; l++) {
    int ni = d->mlp_widths[l], no = d->mlp_widths[l + 1];
    const double *W = p, *b = p + (int64_t)ni * no;
    double *dst = (l == d->mlp_depth - 1) ? out : cur;
    for (int o = 0; o < no; o++) {
      double acc = 0.0;
      for (int i = 0; i < ni; i++) acc += W[(int64_t)o * ni + i] * in[i];
      acc += b[o];
      dst[o] = (l == d->mlp_depth - 1) ? acc : tanh(acc);
    }
    if (l < d->mlp_depth - 1) {
      if (acts) { memcpy(acts + aoff, dst, sizeof(double) * no); aoff += no; }
      in = dst;
      cur = (cur == buf0) ? buf1 : buf0;
    }
    p += (int64_t)ni * no + no;
  }
}

/* VJP of the MLP: gx += J^T g; gP += dOut/dP^T g (if gP). */
static void mlp_vjp(const orc_desc *d, const double *P, const double *x,
                    const double *g, double *gx, double *gP) {
  double acts[MAXW * 8];
  double out[MAXW];
  mlp_forward(d, P, x, out, acts);
  /* offsets of each layer's params and activations */
  int64_t poff[9];
  int aoff[9];
  poff[0] = 0; aoff[0] = 0;
  for (int l = 0; l < d->mlp_depth; l++) {
    int ni = d->mlp_widths[l], no = d->mlp_widths[l + 1];
    poff[l + 1] = poff[l] + (int64_t)ni * no + no;
    aoff[l + 1] = aoff[l] + ((l < d->mlp_depth - 1) ? no : 0);
  }
  double gcur[MAXW], gprev[MAXW];
  int no_last = d->mlp_widths[d->mlp_depth];
  memcpy(gcur, g, sizeof(double) * no_last);
  for (int l = d->mlp_depth - 1; l >= 0; l--) {
    int ni = d->mlp_widths[l], no = d->mlp_widths[l + 1];
    const double *W = P + poff[l];
    const double *xin = (l == 0) ? x : acts + aoff[l - 1];
    /* gcur is dL/d(pre-activation) of layer l. */
    if (gP) {
      double *gW = gP + poff[l], *gb = gW + (int64_t)ni * no;
      for (int o = 0; o < no; o++) {
        for (int i = 0; i < ni; i++) gW[(int64_t)o * ni + i] += gcur[o] * xin[i];
        gb[o] += gcur[o];
      }
    }
    for (int i = 0; i < ni; i++) {
      double acc = 0.0;
      for (int o = 0; o < no; o++) acc += W[(int64_t)o * ni + i] * gcur[o];
      gprev[i] = acc;
    }
    if (l > 0) {
      const double *h = acts + aoff[l - 1];
      for (int i = 0; i < ni; i++) gcur[i] = gprev[i] * (1.0 - h[i] * h[i]);
    } else {
      for (int i = 0; i < ni; i++) gx[i] += gprev[i];
    }
  }
}

static void field_drift(const Field *F, double t, const double *y, double *out) {
  const orc_desc *d = F->d;
  const double *a = F->args;
  switch (d->field) {
    case ORC_LOTKA_VOLTERRA: /* x' = a x - b x y, y' = -c y + d x y */
      out[0] = a[0] * y[0] - a[1] * y[0] * y[1];
      out[1] = -a[2] * y[1] + a[3] * y[0] * y[1];
      break;
    case ORC_VAN_DER_POL: /* x' = y, y' = mu (1 - x^2) y - x */
      out[0] = y[1];
      out[1] = a[0] * (1.0 - y[0] * y[0]) * y[1] - y[0];
      break;
    case ORC_ORNSTEIN_UHLENBECK: /* drift theta (mu - y), args (theta, mu, sigma) */
      for (int i = 0; i < d->dim; i++) out[i] = a[0] * (a[1] - y[i]);
      break;
    case ORC_MLP:
      mlp_forward(d, F->params, y, out, NULL);
      break;
    case ORC_LINEAR:
      for (int i = 0; i < d->dim; i++) {
        double acc = 0.0;
        for (int j = 0; j < d->dim; j++) acc += F->params[i * d->dim + j] * y[j];
        out[i] = acc;
      }
      break;
    case ORC_CALLBACK:
      F->cb(t, y, out, d->dim, F->cb_ctx);
      break;
  }
}

static int64_t diffusion_param_offset(const orc_desc *d) {
  return d->field == ORC_MLP ? mlp_param_count(d) : 0;
}

/* Diagonal diffusion sigma(y) (ControlTerm with a diagonal operator,
 * _term.py:417-427).  OU: sigma constant (args[2]).  TANH_DIAG:
 * sigma = 0.1 tanh(W y + b). */
static void field_diffusion(const Field *F, const double *y, double *sig) {
  const orc_desc *d = F->d;
  if (d->diffusion == ORC_DIFF_OU) {
    for (int i = 0; i < d->dim; i++) sig[i] = F->args[2];
  } else if (d->diffusion == ORC_DIFF_TANH_DIAG) {
    const double *W = F->params + diffusion_param_offset(d);
    const double *b = W + d->dim * d->dim;
    for (int i = 0; i < d->dim; i++) {
      double acc = 0.0;
      for (int j = 0; j < d->dim; j++) acc += W[i * d->dim + j] * y[j];
      sig[i] = 0.1 * tanh(acc + b[i]);
    }
  } else {
    for (int i = 0; i < d->dim; i++) sig[i] = 0.0;
  }
}

/* VJP of the drift: gy += J^T g; gargs += (dF/dargs)^T g; gP += (dF/dP)^T g. */
static void field_drift_vjp(const Field *F, const double *y, const double *g,
                            double *gy, double *gargs, double *gP) {
  const orc_desc *d = F->d;
  const double *a = F->args;
  switch (d->field) {
    case ORC_LOTKA_VOLTERRA:
      gy[0] += g[0] * (a[0] - a[1] * y[1]) + g[1] * (a[3] * y[1]);
      gy[1] += g[0] * (-a[1] * y[0]) + g[1] * (-a[2] + a[3] * y[0]);
      if (gargs) {
        gargs[0] += g[0] * y[0];
        gargs[1] += -g[0] * y[0] * y[1];
        gargs[2] += -g[1] * y[1];
        gargs[3] += g[1] * y[0] * y[1];
      }
      break;
    case ORC_VAN_DER_POL:
      gy[0] += g[1] * (-2.0 * a[0] * y[0] * y[1] - 1.0);
      gy[1] += g[0] + g[1] * a[0] * (1.0 - y[0] * y[0]);
      if (gargs) gargs[0] += g[1] * (1.0 - y[0] * y[0]) * y[1];
      break;
    case ORC_ORNSTEIN_UHLENBECK:
      for (int i = 0; i < d->dim; i++) {
        gy[i] += -a[0] * g[i];
        if (gargs) { gargs[0] += g[i] * (a[1] - y[i]); gargs[1] += g[i] * a[0]; }
      }
      break;
    case ORC_MLP:
      mlp_vjp(d, F->params, y, g, gy, gP);
      break;
    case ORC_LINEAR:
      for (int i = 0; i < d->dim; i++)
        for (int j = 0; j < d->dim; j++) {
          gy[j] += F->params[i * d->dim + j] * g[i];
          if (gP) gP[i * d->dim + j] += g[i] * y[j];
        }
      break;
    default:
      break;
  }
}

/* VJP of y -> sigma(y) * dw (elementwise). */
static void field_diffusion_vjp(const Field *F, const double *y, const double *dw,
                                const double *g, double *gy, double *gargs,
                                double *gP) {
  const orc_desc *d = F->d;
  if (d->diffusion == ORC_DIFF_OU) {
    if (gargs) for (int i = 0; i < d->dim; i++) gargs[2] += g[i] * dw[i];
  } else if (d->diffusion == ORC_DIFF_TANH_DIAG) {
    int64_t off = diffusion_param_offset(d);
    const double *W = F->params + off;
    const double *b = W + d->dim * d->dim;
    for (int i = 0; i < d->dim; i++) {
      double acc = 0.0;
      for (int j = 0; j < d->dim; j++) acc += W[i * d->dim + j] * y[j];
      double th = tanh(acc + b[i]);
      double gz = g[i] * dw[i] * 0.1 * (1.0 - th * th);
      for (int j = 0; j < d->dim; j++) {
        gy[j] += W[i * d->dim + j] * gz;
        if (gP) gP[off + i * d->dim + j] += gz * y[j];
      }
      if (gP) gP[off + d->dim * d->dim + i] += gz;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* One explicit RK step (runge_kutta.py:446-1203, explicit branch).          */
/*                                                                           */
/* k_i = vf(t_i, y_i) * control (+ sigma(y_i) * dW for the SDE MultiTerm,     */
/* _term.py:711-722).  Time is in the direction-normalised coordinate; the    */
/* WrapTerm (_term.py:734-764) evaluates the field at dir * t and multiplies  */
/* the control by dir.                                                       */
/* ------------------------------------------------------------------------ */
typedef struct {
  int dim;
  double k[ORC_MAX_S][64];
  double ystage[ORC_MAX_S][64];
  double y0[64], y1[64], err[64];
  double fsal_f[64];
  double dw[64];
  double tprev, tnext;
} StepOut;

static void rk_step(const Field *F, const Tableau *tab, int dir, double tprev,
                    double tnext, const double *y0, int have_f0, const double *f0,
                    const double *dw, StepOut *so) {
  const orc_desc *d = F->d;
  const int D = d->dim;
  const double dt = tnext - tprev;
  const double control = dir * dt;
  double f[64], sig[64];
  so->dim = D;
  so->tprev = tprev; so->tnext = tnext;
  memcpy(so->y0, y0, sizeof(double) * D);
  if (dw) memcpy(so->dw, dw, sizeof(double) * D);
  for (int i = 0; i < tab->s; i++) {
    double *yi = so->ystage[i];
    if (i == 0) {
      memcpy(yi, y0, sizeof(double) * D);
    } else {
      for (int n = 0; n < D; n++) {
        double inc = 0.0;
        for (int j = 0; j < i; j++) inc += tab->a[i][j] * so->k[j][n];
        yi[n] = y0[n] + inc;
      }
    }
    /* runge_kutta.py:1023: t_i = t1 if c_i == 1 else t0 + c_i dt */
    double ti = (tab->c[i] == 1.0) ? tnext : tprev + tab->c[i] * dt;
    if (i == 0 && have_f0 && tab->fsal) {
      memcpy(f, f0, sizeof(double) * D);
    } else {
      field_drift(F, dir * ti, yi, f);
    }
    if (tab->fsal && i == tab->s - 1) memcpy(so->fsal_f, f, sizeof(double) * D);
    if (d->diffusion != ORC_DIFF_NONE) {
      field_diffusion(F, yi, sig);
      for (int n = 0; n < D; n++) so->k[i][n] = f[n] * control + sig[n] * dw[n];
    } else {
      for (int n = 0; n < D; n++) so->k[i][n] = f[n] * control;
    }
  }
  if (tab->ssal) {
    memcpy(so->y1, so->ystage[tab->s - 1], sizeof(double) * D);
  } else {
    for (int n = 0; n < D; n++) {
      double inc = 0.0;
      for (int j = 0; j < tab->s; j++) inc += tab->b[j] * so->k[j][n];
      so->y1[n] = y0[n] + inc;
    }
  }
  for (int n = 0; n < D; n++) {
    double e = 0.0;
    for (int j = 0; j < tab->s; j++) e += tab->e[j] * so->k[j][n];
    so->err[n] = e;
  }
}

/* One step of an additive-noise stochastic Runge--Kutta method (ShARK,
 * SRA1, SEA) by the additive-noise branch of AbstractSRK.step
 * (srk.py:335-671):
 *   z_j = (y0 + sum_i a_ji h f_i) + g (aw_j W + ah_j H),  f_j = f(t0 + c_j h, z_j),
 *   y1  = (y0 + sum_j b_j h f_j) + g (bw W + bh H),  error = sum_j e_j h f_j.
 * g = g(t0) (the diffusion does not depend on y; the Ornstein-Uhlenbeck and
 * the registered diffusions do not depend on t either, so the correction
 * 0.5 (g(t1) - g(t0)) (W - 2H) of srk.py:607-618 is zero).  The drift's
 * control is the loop's step t1 - t0 (srk.py:364, passed to vf_prod, which
 * the WrapTerm does not flip), not dir * (t1 - t0) as for the RK solvers. */
static void srk_step(const Field *F, const Tableau *tab, int dir, double tprev, double tnext,
                     const double *y0, const double *dw, const double *dh, StepOut *so) {
  const int D = F->d->dim;
  const double h = tnext - tprev;
  double g[64], gw[64], gh[64], f[64];
  so->dim = D;
  so->tprev = tprev; so->tnext = tnext;
  memcpy(so->y0, y0, sizeof(double) * D);
  memcpy(so->dw, dw, sizeof(double) * D);
  field_diffusion(F, y0, g);
  for (int n = 0; n < D; n++) { gw[n] = g[n] * dw[n]; gh[n] = g[n] * dh[n]; }
  for (int j = 0; j < tab->s; j++) {
    double *z = so->ystage[j];
    for (int n = 0; n < D; n++) {
      double drift = 0.0;
      for (int i = 0; i < j; i++) drift += tab->a[j][i] * so->k[i][n];
      z[n] = (y0[n] + drift) + (tab->aw[j] * gw[n] + tab->ah[j] * gh[n]);
    }
    field_drift(F, dir * (tprev + tab->c[j] * h), z, f);
    for (int n = 0; n < D; n++) so->k[j][n] = f[n] * h;
  }
  for (int n = 0; n < D; n++) {
    double drift = 0.0, e = 0.0;
    for (int j = 0; j < tab->s; j++) {
      drift += tab->b[j] * so->k[j][n];
      e += tab->e[j] * so->k[j][n];
    }
    so->y1[n] = (y0[n] + drift) + (tab->bw * gw[n] + tab->bh * gh[n]);
    so->err[n] = e;
  }
}

/* ------------------------------------------------------------------------ */
/* Dense interpolation inside the step just taken.                           */
/* ------------------------------------------------------------------------ */
/* linear_rescale (_misc.py:71-82) */
static double linear_rescale(double t0, double t, double t1) {
  if (t0 == t1) return 0.0;
  return (t - t0) / (t1 - t0);
}

/* Tsit5 interpolation weights b_i(theta) (tsit5.py:119-150). */
static void tsit5_weights(double t, double w[7]) {
  w[0] = -1.0530884977290216 * t * (t - 1.3299890189751412) *
         (t * t - 1.4364028541716351 * t + 0.7139816917074209);
  w[1] = 0.1017 * t * t * (t * t - 2.1966568338249754 * t + 1.2949852507374631);
  w[2] = 2.490627285651252793 * t * t * (t * t - 2.38535645472061657 * t + 1.57803468208092486);
  w[3] = -16.54810288924490272 * (t - 1.21712927295533244) * (t - 0.61620406037800089) * t * t;
  w[4] = 47.37952196281928122 * (t - 1.203071208372362603) * (t - 0.658047292653547382) * t * t;
  w[5] = -34.87065786149660974 * (t - 1.2) * (t - 0.666666666666666667) * t * t;
  w[6] = 2.5 * (t - 1) * (t - 0.6) * t * t;
}

/* Dopri8 dense-output weights theta P_j(theta), or their theta-derivative
 * P_j + theta P_j' (deriv = 1). */
static void dopri8_weights(double t, double w[ORC_MAX_S], int deriv) {
  for (int j = 0; j < 14; j++) {
    const double *c = DOPRI8_P[j];
    double p = ((((c[0] * t + c[1]) * t + c[2]) * t + c[3]) * t + c[4]) * t + c[5];
    if (deriv) {
      double dp = (((5 * c[0] * t + 4 * c[1]) * t + 3 * c[2]) * t + 2 * c[3]) * t + c[4];
      w[j] = p + t * dp;
    } else {
      w[j] = t * p;
    }
  }
}

/* Coefficients of the interpolant as a linear map of (y0, y1, k_j):
 * out = ay0 * y0 + ay1 * y1 + sum_j g[j] k_j.  Used by the VJP. */
static void interp_linear_coeffs(int solver, int s, double th, double *ay0,
                                 double *ay1, double g[ORC_MAX_S]) {
  for (int j = 0; j < ORC_MAX_S; j++) g[j] = 0.0;
  double t2 = th * th, t3 = t2 * th, t4 = t3 * th;
  switch (solver) {
    case ORC_TSIT5:
      *ay0 = 1.0; *ay1 = 0.0; tsit5_weights(th, g);
      break;
    case ORC_DOPRI8:
      *ay0 = 1.0; *ay1 = 0.0; dopri8_weights(th, g, 0);
      break;
    case ORC_DOPRI5: {
      /* _local_interpolation.py:109-127 expanded in the monomials. */
      double M = 16 * t4 - 32 * t3 + 16 * t2;
      *ay0 = -8 * t4 + 18 * t3 - 11 * t2 + 1 + M;
      *ay1 = -8 * t4 + 14 * t3 - 5 * t2;
      for (int j = 0; j < 7; j++) g[j] = M * DOPRI5_CMID[j];
      g[0] += -2 * t4 + 5 * t3 - 4 * t2 + th;
      g[6] += 2 * t4 - 3 * t3 + t2;
      break;
    }
    case ORC_HEUN: /* _local_interpolation.py:61-66 */
      *ay0 = 2 * t3 - 3 * t2 + 1;
      *ay1 = -2 * t3 + 3 * t2;
      g[0] = t3 - 2 * t2 + th;
      g[s - 1] = t3 - t2;
      break;
    default: /* Euler: LocalLinearInterpolation */
      *ay0 = 1.0 - th; *ay1 = th;
      break;
  }
}

/* Forward evaluation, following the reference's evaluation order. */
static void interp_eval(int solver, const StepOut *so, int s, double t, double *out) {
  const int D = so->dim;
  double th = linear_rescale(so->tprev, t, so->tnext);
  switch (solver) {
    case ORC_TSIT5: {
      double w[7];
      tsit5_weights(th, w);
      for (int n = 0; n < D; n++) {
        double acc = 0.0;
        for (int j = 0; j < 7; j++) acc += w[j] * so->k[j][n];
        out[n] = so->y0[n] + acc;
      }
      break;
    }
    case ORC_DOPRI8: {
      double w[ORC_MAX_S];
      dopri8_weights(th, w, 0);
      for (int n = 0; n < D; n++) {
        double acc = 0.0;
        for (int j = 0; j < 14; j++) acc += w[j] * so->k[j][n];
        out[n] = so->y0[n] + acc;
      }
      break;
    }
    case ORC_DOPRI5:
      for (int n = 0; n < D; n++) {
        double cm = 0.0;
        for (int j = 0; j < 7; j++) cm += DOPRI5_CMID[j] * so->k[j][n];
        double y0 = so->y0[n], y1 = so->y1[n], ymid = y0 + cm;
        double f0 = so->k[0][n], f1 = so->k[6][n];
        double a = 2 * (f1 - f0) - 8 * (y1 + y0) + 16 * ymid;
        double b = 5 * f0 - 3 * f1 + 18 * y0 + 14 * y1 - 32 * ymid;
        double c = f1 - 4 * f0 - 11 * y0 - 5 * y1 + 16 * ymid;
        out[n] = (((a * th + b) * th + c) * th + f0) * th + y0;
      }
      break;
    case ORC_HEUN:
      for (int n = 0; n < D; n++) {
        double y0 = so->y0[n], y1 = so->y1[n], k0 = so->k[0][n], k1 = so->k[s - 1][n];
        double a = k0 + k1 + 2 * y0 - 2 * y1;
        double b = -2 * k0 - k1 - 3 * y0 + 3 * y1;
        out[n] = ((a * th + b) * th + k0) * th + y0;
      }
      break;
    default:
      for (int n = 0; n < D; n++) out[n] = so->y0[n] + th * (so->y1[n] - so->y0[n]);
      break;
  }
}

/* ------------------------------------------------------------------------ */
/* Step-size controllers.                                                    */
/* ------------------------------------------------------------------------ */
typedef struct {
  /* PID (pid.py:388-392) */
  double prev_inv, prev_prev_inv;
  int at_dtmin;
  /* Constant (constant.py:41-57) */
  int steps_completed, num_steps;
  double t0_sim, t1_sim;
} CtrlState;

static double prevbefore(double x) { return nextafter(x, -INFINITY); }

/* optx.rms_norm: two_norm / sqrt(size). */
static double rms_norm(const double *x, int n) {
  double acc = 0.0;
  for (int i = 0; i < n; i++) acc += x[i] * x[i];
  return sqrt(acc) / sqrt((double)n);
}

/* PIDController.adapt_step_size (pid.py:394-567).  `scaled` is precomputed by
 * the caller because the backsolve adjoint uses a different norm. */
static int pid_adapt(const orc_desc *d, double error_order, double t0, double t1,
                     double scaled, CtrlState *cs, double *next_t0, double *next_t1,
                     int *result) {
  int has_dtmin = !isnan(d->dtmin), has_dtmax = !isnan(d->dtmax);
  int keep = scaled < 1.0;
  if (has_dtmin) keep = keep | cs->at_dtmin;
  double prev_dt = t1 - t0;
  double inv = 1.0 / scaled;
  double c1 = (d->icoeff + d->pcoeff + d->dcoeff) / error_order;
  double c2 = -(d->pcoeff + 2 * d->dcoeff) / error_order;
  double c3 = d->dcoeff / error_order;
  double f1 = (c1 == 0) ? 1.0 : pow(inv, c1);
  double f2 = (c2 == 0) ? 1.0 : pow(cs->prev_inv, c2);
  double f3 = (c3 == 0) ? 1.0 : pow(cs->prev_prev_inv, c3);
  double fmin = keep ? 1.0 : d->factormin;
  double fmax = keep ? d->factormax : d->safety;
  double factor = d->safety * f1 * f2 * f3;
  factor = fmax < (factor > fmin ? factor : fmin) ? fmax : (factor > fmin ? factor : fmin);
  double dt = prev_dt * factor;
  if (inv == 0.0 || isinf(inv)) inv = 1.0;
  *result = ORC_SUCCESSFUL;
  if (has_dtmax) dt = dt < d->dtmax ? dt : d->dtmax;
  int at_dtmin = cs->at_dtmin;
  if (has_dtmin) {
    if (!d->force_dtmin && dt < d->dtmin) *result = ORC_DT_MIN_REACHED;
    if (at_dtmin && factor == 1.0) dt = d->dtmin;
    at_dtmin = dt <= d->dtmin;
    dt = dt > d->dtmin ? dt : d->dtmin;
  }
  *next_t0 = keep ? t1 : t0;
  *next_t1 = *next_t0 + dt;
  double new_inv = keep ? inv : cs->prev_inv;
  double new_prev = keep ? cs->prev_inv : cs->prev_prev_inv;
  cs->prev_inv = new_inv;
  cs->prev_prev_inv = new_prev;
  cs->at_dtmin = at_dtmin;
  return keep;
}

/* ConstantStepSize.adapt_step_size (constant.py:59-104). */
static int constant_adapt(double t1, CtrlState *cs, double *next_t0, double *next_t1) {
  int sc = cs->steps_completed + 1;
  double t1n = cs->t0_sim + (cs->t1_sim - cs->t0_sim) * ((double)sc / (double)cs->num_steps);
  if (sc == cs->num_steps) t1n = cs->t1_sim;
  /* an infinite t1 (num_steps = -1) keeps adding dt0 (constant.py:48-55, 94-97) */
  if (cs->num_steps < 0) t1n = t1 + cs->t1_sim;
  cs->steps_completed = sc;
  *next_t0 = t1;
  *next_t1 = t1n;
  return 1;
}

/* ClipStepSizeController (clip.py).  `ts` holds n times sorted increasing in
 * the caller's time; the controller works in the loop's direction-flipped
 * time, where the sorted array is sort(ts * direction) (clip.py:203-213). */
static double clip_get(const double *ts, int n, int i, int dir) {
  /* _get_t (clip.py:55-62): ts[i], +inf past the end */
  if (i >= n) return INFINITY;
  return dir > 0 ? ts[i] : -ts[n - 1 - i];
}

/* _find_idx_with_hint (clip.py:102-118): the first index whose time is
 * strictly greater than t, by a linear search from the hint. */
static int clip_find(const double *ts, int n, int dir, double t, int hint) {
  int i = hint;
  while (i < n && clip_get(ts, n, i, dir) <= t) i++;
  while (i > 0 && clip_get(ts, n, i - 1, dir) > t) i--;
  return i;
}

/* _bump_next_t0 (clip.py:79-99): a step that ended at prevbefore(x) or at x
 * for x in ts restarts after x (two nextafters, or one). */
static double clip_bump(const double *ts, int n, int dir, double t, int *made_jump) {
  double n1 = nextafter(t, INFINITY);
  int mj1 = 0, mj2 = 0;
  for (int i = 0; i < n; i++) {
    double v = clip_get(ts, n, i, dir);
    mj1 |= (v == n1);
    mj2 |= (v == t);
  }
  double out = mj1 ? nextafter(n1, INFINITY) : t;
  if (mj2) out = n1;
  *made_jump = mj1 | mj2;
  return out;
}

typedef struct {
  const double *step_ts, *jump_ts;
  int n_step, n_jump, step_index, jump_index;
} ClipState;

/* jnp.sign, with NaN for NaN */
static double ev_sign(double x) { return isnan(x) ? NAN : (double)((x > 0) - (x < 0)); }

/* ClipStepSizeController.init (clip.py:215-276): the first step end clipped
 * to the first step time after t0 and to just before the first jump. */
static double clip_init(ClipState *c, int dir, double t0, double tnext) {
  if (c->n_step) {
    c->step_index = clip_find(c->step_ts, c->n_step, dir, t0, 0);
    double v = clip_get(c->step_ts, c->n_step, c->step_index, dir);
    tnext = v < tnext ? v : tnext;
  }
  if (c->n_jump) {
    c->jump_index = clip_find(c->jump_ts, c->n_jump, dir, t0, 0);
    double v = nextafter(clip_get(c->jump_ts, c->n_jump, c->jump_index, dir), -INFINITY);
    tnext = v < tnext ? v : tnext;
  }
  return tnext;
}

/* ClipStepSizeController.adapt_step_size after the inner controller
 * (clip.py:330-389).  Returns made_jump. */
static int clip_adapt(ClipState *c, int dir, double *next_t0, double *next_t1) {
  int made_jump = 0, mj;
  if (c->n_step) {
    double b0 = clip_bump(c->step_ts, c->n_step, dir, *next_t0, &mj);
    c->step_index = clip_find(c->step_ts, c->n_step, dir, b0, c->step_index);
    double v = clip_get(c->step_ts, c->n_step, c->step_index, dir);
    if (v < *next_t1) *next_t1 = v;
  }
  if (c->n_jump) {
    *next_t0 = clip_bump(c->jump_ts, c->n_jump, dir, *next_t0, &mj);
    double lo = nextafter(*next_t0, INFINITY);
    if (lo > *next_t1) *next_t1 = lo;
    made_jump |= mj;
    c->jump_index = clip_find(c->jump_ts, c->n_jump, dir, *next_t0, c->jump_index);
    double v = nextafter(clip_get(c->jump_ts, c->n_jump, c->jump_index, dir), -INFINITY);
    if (v < *next_t1) *next_t1 = v;
  }
  return made_jump;
}

static double error_order_of(const orc_desc *d, const Tableau *tab) {
  if (d->error_order > 0) return d->error_order;
  if (d->diffusion != ORC_DIFF_NONE) return tab->strong_order + 0.5;
  return (double)tab->order;
}

/* ------------------------------------------------------------------------ */
/* Events (_event.py, _integrate.py:542-633, 686-821).                       */
/* ------------------------------------------------------------------------ */
static void interp_eval(int solver, const StepOut *so, int s, double t, double *out);
static void interp_deriv_coeffs(int solver, int s, double t, double *ay0, double *ay1,
                                double g[ORC_MAX_S]);

/* Value of condition i at the loop's time t (the direction-flipped time the
 * reference passes to cond_fn) and state y; booleans are 0 / 1. */
static double ev_value(const Field *F, int dir, int i, double t, const double *y) {
  const orc_desc *d = F->d;
  const double *c = d->ev_coef + 6 * i;
  if (d->ev_kind[i] == ORC_EV_STEADY) {
    /* norm(vf) < atol + rtol norm(y) with the PID's rms_norm; the wrapped
     * field is dir * f(dir * t, y), of the same norm (_event.py:164-175) */
    double f[64];
    field_drift(F, dir * t, y, f);
    return rms_norm(f, d->dim) < c[1] + c[0] * rms_norm(y, d->dim) ? 1.0 : 0.0;
  }
  /* at most four state coefficients: components 0 .. min(dim, 4) - 1 */
  double v = 0.0;
  for (int n = 0; n < (d->dim < 4 ? d->dim : 4); n++) v += c[n] * y[n];
  v += c[4] * t;
  v += c[5];
  if (d->ev_kind[i] == ORC_EV_LINEAR_BOOL) return v > 0 ? 1.0 : 0.0;
  return v;
}

/* Whether condition i triggers between values old and new (_integrate.py:585-602). */
static int ev_triggered(const orc_desc *d, int i, double old_v, double new_v) {
  if (d->ev_kind[i] != ORC_EV_LINEAR) return new_v != 0.0;
  double so = ev_sign(old_v), sn = ev_sign(new_v);
  switch (d->ev_dir[i]) {
    case ORC_EV_UP: return so <= 0 && sn > 0;
    case ORC_EV_DOWN: return so > 0 && sn <= 0;
    default: return so != sn || isnan(so) || isnan(sn);
  }
}

/* The event's root find (_integrate.py:704-779): optimistix.Newton with
 * cauchy_termination on g(t) = cond_i(t, interp(t)) over the last step's
 * interval [so->tprev, so->tnext] from t = so->tnext, each iterate clipped to
 * the interval; it stops once the step was below atol + rtol |t| and |g| at
 * the previous iterate below atol, from the second iteration on, or after 256
 * iterations (not converged).  A boolean condition has its root at the end of
 * the step.  Returns the root; *ok = 0 if it did not converge. */
static double ev_root(const Field *F, const Tableau *tab, int i, const StepOut *so, int *ok) {
  const orc_desc *d = F->d;
  const int D = d->dim < 4 ? d->dim : 4; /* the condition's state coefficients */
  *ok = 1;
  if (d->ev_kind[i] != ORC_EV_LINEAR) return so->tnext;
  const double *c = d->ev_coef + 6 * i;
  const double lo = so->tprev, hi = so->tnext, span = hi - lo;
  double y = hi;
  for (int step = 1; step <= 256; step++) {
    double yv[64], ay0, ay1, g[ORC_MAX_S];
    interp_eval(d->solver, so, tab->s, y, yv);
    double f = 0.0;
    for (int n = 0; n < D; n++) f += c[n] * yv[n];
    f += c[4] * y;
    f += c[5];
    /* g'(t) = w . dinterp/dt + wt, dinterp/dt = (d/dtheta) / span */
    interp_deriv_coeffs(d->solver, tab->s, linear_rescale(lo, y, hi), &ay0, &ay1, g);
    double fp = 0.0;
    for (int n = 0; n < D; n++) {
      double v = ay0 * so->y0[n] + ay1 * so->y1[n];
      for (int j = 0; j < tab->s; j++) v += g[j] * so->k[j][n];
      fp += c[n] * (span == 0.0 ? 0.0 : v / span);
    }
    fp += c[4];
    double diff = f / fp;
    double ny = y - diff;
    if (ny < lo) ny = lo;
    if (ny > hi) ny = hi;
    if (isnan(ny)) { *ok = 0; return y; }
    double diffsize = fabs(diff) / (d->newton_atol + d->newton_rtol * fabs(ny));
    y = ny;
    if (step >= 2 && diffsize < 1.0 && fabs(f) < d->newton_atol) return y;
  }
  *ok = 0;
  return y;
}

/* ------------------------------------------------------------------------ */
/* The per-trajectory solve loop (_integrate.py:302-885, init 1036-1305).    */
/* ------------------------------------------------------------------------ */
typedef struct {
  /* inputs */
  const orc_desc *d;
  const double *t0, *t1, *dt0; /* dt0 may be NULL (None) */
  int64_t time_stride;
  const double *y0;
  const double *args;
  int64_t args_stride;
  const double *params;
  const double *ts;
  orc_vf_cb cb;
  void *cb_ctx;
  /* outputs */
  double *ys_out, *ts_out;
  int32_t *result, *stats;
  /* SaveAt(dense=True): step times [B, max_steps + 1] (the direction-flipped
   * frame of the loop, +inf where unused), per accepted step (y0, y1, k_0..k_{s-1})
   * [B, max_steps, (2 + s) dim] (+inf where unused), and steps + 1 [B] */
  double *dense_ts, *dense_info;
  int32_t *dense_n;
  /* Event: the index of the condition that ended the solve, -1 if none [B] */
  int32_t *event_index;
  /* Resuming (_integrate.py:1252-1271, 1489-1500): per trajectory a record
   * of ORC_STATE_HEAD + dim doubles -- the controller state (PID: prev_inv,
   * prev_prev_inv, at_dtmin, 0; constant: steps_completed, num_steps, t0,
   * t1 or dt0, in the direction-flipped time), whether a controller state is
   * given, the solver state's first_step, made_jump, and the FSAL value f0.
   * state_in NULL: a fresh solve; state_out NULL: not reported. */
  const double *state_in;
  double *state_out;
} SolveIO;

#define ORC_STATE_HEAD 7

/* A record of one accepted step, kept for the discretise-then-optimise VJP. */
typedef struct {
  double tprev, tnext;
  int save_lo, save_hi; /* save indices [lo, hi) produced by this step */
} TapeStep;

typedef struct {
  TapeStep *steps;
  double *ys;  /* y at the start of each accepted step [n x D] */
  int n, cap;
  int dir;
  int t0_eq_t1;
  int t1_slot;
} Tape;

static void tape_push(Tape *tp, int D, double tprev, double tnext, const double *y,
                      int lo, int hi) {
  if (tp->n == tp->cap) {
    tp->cap = tp->cap ? tp->cap * 2 : 64;
    tp->steps = (TapeStep *)realloc(tp->steps, sizeof(TapeStep) * tp->cap);
    tp->ys = (double *)realloc(tp->ys, sizeof(double) * D * tp->cap);
  }
  tp->steps[tp->n].tprev = tprev;
  tp->steps[tp->n].tnext = tnext;
  tp->steps[tp->n].save_lo = lo;
  tp->steps[tp->n].save_hi = hi;
  memcpy(tp->ys + (int64_t)tp->n * D, y, sizeof(double) * D);
  tp->n++;
}

/* Output size of a SaveAt (_integrate.py:1273-1293). */
static int n_save_of(const orc_desc *d) {
  int n = (d->save_t0 ? 1 : 0) + d->n_ts;
  if (d->save_steps > 0) n += d->max_steps / d->save_steps;
  if (d->save_t1 && (d->save_steps == 0 || d->max_steps % d->save_steps != 0)) n += 1;
  return n;
}

/* Dense info record length of one accepted step: (y0, y1, k_0..k_{s-1}). */
static int dense_rec_of(const orc_desc *d) { return (2 + tableau_of(d->solver)->s) * d->dim; }

static void solve_one(const SolveIO *io, int64_t bidx, Tape *tape) {
  const orc_desc *d = io->d;
  const Tableau *tab = tableau_of(d->solver);
  const int D = d->dim;
  const int n_save = n_save_of(d);
  Field F = {d, io->args + bidx * io->args_stride, io->params, io->cb, io->cb_ctx};
  double *ys = io->ys_out + bidx * (int64_t)n_save * D;
  double *tso = io->ts_out + bidx * (int64_t)n_save;
  for (int64_t i = 0; i < (int64_t)n_save * D; i++) ys[i] = INFINITY;
  for (int i = 0; i < n_save; i++) tso[i] = INFINITY;

  double t0 = io->t0[bidx * io->time_stride], t1 = io->t1[bidx * io->time_stride];
  /* _integrate.py:1157-1166: direction = where(t0 < t1, 1, -1) */
  int dir = (t0 < t1) ? 1 : -1;
  t0 *= dir; t1 *= dir;
  int has_dt0 = io->dt0 != NULL;
  double dt0 = has_dt0 ? io->dt0[bidx * io->time_stride] * dir : 0.0;
  double y[64];
  memcpy(y, io->y0 + bidx * D, sizeof(double) * D);
  if (tape) { tape->dir = dir; tape->t0_eq_t1 = (t0 == t1); }

  /* controller init (pid.py:316-392, constant.py:30-57, clip.py:215-276) */
  CtrlState cs;
  memset(&cs, 0, sizeof cs);
  ClipState clip = {io->ts + d->n_ts, io->ts + d->n_ts + d->n_step_ts, d->n_step_ts,
                    d->n_jump_ts, 0, 0};
  const int clipping = d->n_step_ts > 0 || d->n_jump_ts > 0;
  double tnext;
  if (d->controller == ORC_PID) {
    /* The terms are already wrapped when init runs (_integrate.py:1172-1176,
     * 1254), so _select_initial_step returns 0.01 (pid.py:48-49). */
    double h = has_dt0 ? dt0 : 0.01;
    if (!isnan(d->dtmax)) h = h < d->dtmax ? h : d->dtmax;
    if (!isnan(d->dtmin)) h = h > d->dtmin ? h : d->dtmin;
    tnext = t0 + h;
    cs.prev_inv = 1.0; cs.prev_prev_inv = 1.0; cs.at_dtmin = 0;
    if (clipping) tnext = clip_init(&clip, dir, t0, tnext);
  } else {
    cs.steps_completed = 1;
    cs.num_steps = isfinite(t1) ? (int)ceil((t1 - t0) / nextafter(dt0, INFINITY)) : -1;
    cs.t0_sim = t0; cs.t1_sim = isfinite(t1) ? t1 : dt0;
    tnext = t0 + dt0;
  }
  /* a passed controller state replaces the controller's init; the first
   * step is then t0 + dt0, unclipped (dt0=None keeps the initial step) */
  const double *st_in = io->state_in ? io->state_in + bidx * (int64_t)(ORC_STATE_HEAD + D)
                                     : NULL;
  if (st_in && st_in[4] != 0.0) {
    if (d->controller == ORC_PID) {
      cs.prev_inv = st_in[0];
      cs.prev_prev_inv = st_in[1];
      cs.at_dtmin = st_in[2] != 0.0;
      if (has_dt0) tnext = t0 + dt0;
    } else {
      cs.steps_completed = (int)st_in[0];
      cs.num_steps = (int)st_in[1];
      cs.t0_sim = st_in[2];
      cs.t1_sim = st_in[3];
    }
  }
  tnext = tnext < t1 ? tnext : t1;
  double tprev = t0;
  double t1_clip_floor = t1;
  for (int i = 0; i < 100; i++) t1_clip_floor = prevbefore(t1_clip_floor);
  const double eord = error_order_of(d, tab);

  int save_index = 0, ts_index = 0;
  if (d->save_t0) {
    for (int n = 0; n < D; n++) ys[n] = y[n];
    tso[0] = t0;
    save_index = 1;
  }
  /* SaveAt(dense=True): buffers full of inf, dense_ts[0] = t0 (_integrate.py:324-327,
   * 1315-1323) */
  const int drec = dense_rec_of(d);
  double *dts = NULL, *dinf = NULL;
  if (io->dense_ts) {
    dts = io->dense_ts + bidx * (int64_t)(d->max_steps + 1);
    dinf = io->dense_info + bidx * (int64_t)d->max_steps * drec;
    for (int i = 0; i <= d->max_steps; i++) dts[i] = INFINITY;
    for (int64_t i = 0; i < (int64_t)d->max_steps * drec; i++) dinf[i] = INFINITY;
    dts[0] = t0;
  }
  int first_step = 1;
  int made_jump = 0; /* _integrate.py:1309, 425 */
  double f0[64];
  memset(f0, 0, sizeof f0);
  if (st_in) { /* a passed solver state and made_jump */
    made_jump = st_in[6] != 0.0;
    if (tab->fsal && st_in[5] == 0.0) {
      first_step = 0;
      memcpy(f0, st_in + ORC_STATE_HEAD, sizeof(double) * D);
    }
  }
  int result = ORC_SUCCESSFUL;
  int num_steps = 0, num_acc = 0, num_rej = 0;
  StepOut so;
  double dw[64], dh[64];
  /* Event values at (t0, y0) (_integrate.py:1333-1426): a boolean condition
   * that already holds ends the solve before its first step. */
  double ev_val[ORC_MAX_EVENTS];
  int ev_idx = -1, ev_have = 0;
  StepOut ev_so; /* the step over which the event fired */
  for (int i = 0; i < d->n_event; i++) {
    ev_val[i] = ev_value(&F, dir, i, t0, y);
    if (ev_idx < 0 && d->ev_kind[i] != ORC_EV_LINEAR && ev_val[i] != 0.0) ev_idx = i;
  }
  if (ev_idx >= 0) result = ORC_EVENT_OCCURRED;
  while (tprev < t1 && result == ORC_SUCCESSFUL) {
    if (num_steps >= d->max_steps) break;
    const double *dwp = NULL;
    if (d->diffusion != ORC_DIFF_NONE) {
      step_increment(d, (uint32_t)bidx, dir, tprev, tnext, dw, dh);
      dwp = dw;
    }
    if (ORC_IS_SRK(d->solver)) {
      srk_step(&F, tab, dir, tprev, tnext, y, dw, dh, &so);
    } else {
      /* FSAL reuse unless first step or just after a jump (runge_kutta.py:684-700) */
      rk_step(&F, tab, dir, tprev, tnext, y, !(first_step || made_jump), f0, dwp, &so);
    }
    for (int n = 0; n < D; n++)
      if (isnan(so.err[n])) so.err[n] = INFINITY; /* _integrate.py:386 */
    int keep, cres = ORC_SUCCESSFUL;
    double nt0, nt1;
    if (d->controller == ORC_PID) {
      /* pid.py:466-492: scale against max(|y0|, |y1|), y1 replaced by y0 if NaN */
      int any_nan = 0;
      for (int n = 0; n < D; n++) any_nan |= isnan(so.y1[n]);
      double sc[64];
      for (int n = 0; n < D; n++) {
        double a0 = fabs(y[n]), a1 = fabs(any_nan ? y[n] : so.y1[n]);
        double ym = a0 > a1 ? a0 : a1;
        sc[n] = so.err[n] / (d->atol + ym * d->rtol);
      }
      double scaled = rms_norm(sc, D);
      keep = pid_adapt(d, eord, tprev, tnext, scaled, &cs, &nt0, &nt1, &cres);
      if (clipping) {
        int mj = clip_adapt(&clip, dir, &nt0, &nt1);
        if (keep) made_jump = mj; /* a rejected step keeps the old flag (:425) */
      }
    } else {
      keep = constant_adapt(tnext, &cs, &nt0, &nt1);
    }
    /* _integrate.py:410-413 */
    nt0 = nt0 < t1 ? nt0 : t1;
    if (nt1 > t1_clip_floor) nt1 = keep ? t1 : nt0 + 0.5 * (t1 - nt0);
    if (keep) {
      int lo = save_index;
      /* _integrate.py:456-487: save every ts <= tnext of the step just taken */
      while (ts_index < d->n_ts && dir * io->ts[ts_index] <= tnext) {
        interp_eval(d->solver, &so, tab->s, dir * io->ts[ts_index], ys + (int64_t)save_index * D);
        tso[save_index] = dir * io->ts[ts_index];
        ts_index++; save_index++;
      }
      /* _integrate.py:493-527: SaveAt(steps=n) saves (tnext, y1) of every n-th
       * accepted step, after the ts of the step */
      if (d->save_steps > 0 && (num_acc + 1) % d->save_steps == 0) {
        for (int n = 0; n < D; n++) ys[(int64_t)save_index * D + n] = so.y1[n];
        tso[save_index] = tnext;
        save_index++;
      }
      /* _integrate.py:529-540: the step's dense info and its end time */
      if (dts) {
        dts[num_acc + 1] = tnext;
        double *r = dinf + (int64_t)num_acc * drec;
        memcpy(r, y, sizeof(double) * D);
        memcpy(r + D, so.y1, sizeof(double) * D);
        for (int j = 0; j < tab->s; j++) memcpy(r + (2 + j) * D, so.k[j], sizeof(double) * D);
      }
      if (tape) tape_push(tape, D, tprev, tnext, y, lo, save_index);
      memcpy(y, so.y1, sizeof(double) * D);
      if (tab->fsal) { memcpy(f0, so.fsal_f, sizeof(double) * D); first_step = 0; }
    }
    if (result == ORC_SUCCESSFUL) result = cres;
    num_steps++;
    if (keep) num_acc++; else num_rej++;
    tprev = nt0;
    tnext = nt1;
    /* _integrate.py:542-633: every condition at the new (tprev, y); the first
     * that triggered (in order) ends the solve */
    if (d->n_event) {
      int fired = -1;
      for (int i = 0; i < d->n_event; i++) {
        double v = ev_value(&F, dir, i, tprev, y);
        if (fired < 0 && ev_triggered(d, i, ev_val[i], v)) fired = i;
        ev_val[i] = v;
      }
      if (fired >= 0) {
        ev_idx = fired;
        ev_so = so;
        ev_have = 1;
        result = ORC_EVENT_OCCURRED;
      }
    }
  }
  /* _integrate.py:686-821: with a root finder the final time is the event's
   * root inside the last step and y there its interpolant (y itself when no
   * step was taken); every save after it is deleted */
  double tfinal = tprev, yf[64];
  const double *yfinal = y;
  const int ev_root_finder = d->n_event > 0 && d->event_root;
  if (ev_root_finder && ev_idx >= 0) {
    if (ev_have) {
      int ok = 1;
      tfinal = ev_root(&F, tab, ev_idx, &ev_so, &ok);
      interp_eval(d->solver, &ev_so, tab->s, tfinal, yf);
      yfinal = yf;
      if (!ok) result = ORC_EVENT_ROOT_MAX_STEPS;
    }
    for (int i = 0; i < n_save; i++) {
      if (tso[i] > tfinal) {
        if (tso[i] < INFINITY) save_index--;
        tso[i] = INFINITY;
        for (int n = 0; n < D; n++) ys[(int64_t)i * D + n] = INFINITY;
      }
    }
  }
  /* _integrate.py:823-845: t0 == t1 fills the ts outputs with y0 */
  if (t0 == t1) {
    for (int i = 0; i < d->n_ts; i++) {
      for (int n = 0; n < D; n++) ys[(int64_t)save_index * D + n] = yfinal[n];
      tso[save_index] = t0;
      save_index++;
    }
  }
  /* _integrate.py:847-877: the t1 save goes to the next free slot, unless
   * SaveAt(steps=n) saved it: always for n = 1, for n > 1 when the accepted
   * steps are a multiple of n */
  int t1_via_steps = d->save_steps == 0 ? 0 : (d->save_steps == 1 ? 1 : (num_acc % d->save_steps == 0));
  /* with an event root finder the final value is saved whenever steps saved
   * the t1 value, since that save was deleted above (:866-872) */
  const int save_final = ev_root_finder ? (d->save_t1 || t1_via_steps)
                                        : (d->save_t1 && !t1_via_steps);
  if (save_final) {
    for (int n = 0; n < D; n++) ys[(int64_t)save_index * D + n] = yfinal[n];
    tso[save_index] = tfinal;
    if (tape) tape->t1_slot = save_index;
    save_index++;
  }
  if (result == ORC_SUCCESSFUL && tprev < t1) result = ORC_MAX_STEPS_REACHED;
  for (int i = 0; i < n_save; i++) tso[i] *= dir;
  if (io->state_out) { /* SaveAt(controller_state, solver_state, made_jump) */
    double *so_ = io->state_out + bidx * (int64_t)(ORC_STATE_HEAD + D);
    if (d->controller == ORC_PID) {
      so_[0] = cs.prev_inv; so_[1] = cs.prev_prev_inv; so_[2] = cs.at_dtmin; so_[3] = 0.0;
    } else {
      so_[0] = cs.steps_completed; so_[1] = cs.num_steps; so_[2] = cs.t0_sim; so_[3] = cs.t1_sim;
    }
    const int fsal_valid = tab->fsal && !first_step;
    so_[4] = 1.0;
    so_[5] = fsal_valid ? 0.0 : 1.0;
    so_[6] = made_jump;
    for (int n = 0; n < D; n++) so_[ORC_STATE_HEAD + n] = fsal_valid ? f0[n] : 0.0;
  }
  io->result[bidx] = result;
  if (io->dense_n) io->dense_n[bidx] = num_acc + 1;
  if (io->event_index) io->event_index[bidx] = ev_idx;
  io->stats[bidx * 3 + 0] = num_steps;
  io->stats[bidx * 3 + 1] = num_acc;
  io->stats[bidx * 3 + 2] = num_rej;
}

static void validate_desc(const orc_desc *d) { (void)d; init_tableaus(); }

int orc_solve_state(const orc_desc *d, int64_t B, const double *t0, const double *t1,
                    const double *dt0, int64_t time_stride, const double *y0,
                    const double *args, int64_t args_stride, const double *params,
                    const double *ts, orc_vf_cb cb, void *cb_ctx, double *ys_out,
                    double *ts_out, int32_t *result, int32_t *stats, double *dense_ts,
                    double *dense_info, int32_t *dense_n, int32_t *event_index,
                    const double *state_in, double *state_out, int nthreads);

int orc_solve_dense(const orc_desc *d, int64_t B, const double *t0, const double *t1,
                    const double *dt0, int64_t time_stride, const double *y0,
                    const double *args, int64_t args_stride, const double *params,
                    const double *ts, orc_vf_cb cb, void *cb_ctx, double *ys_out,
                    double *ts_out, int32_t *result, int32_t *stats, double *dense_ts,
                    double *dense_info, int32_t *dense_n, int32_t *event_index,
                    int nthreads) {
  return orc_solve_state(d, B, t0, t1, dt0, time_stride, y0, args, args_stride, params, ts, cb,
                         cb_ctx, ys_out, ts_out, result, stats, dense_ts, dense_info, dense_n,
                         event_index, NULL, NULL, nthreads);
}

/* orc_solve_dense with the resume records (SolveIO.state_in / state_out). */
int orc_solve_state(const orc_desc *d, int64_t B, const double *t0, const double *t1,
                    const double *dt0, int64_t time_stride, const double *y0,
                    const double *args, int64_t args_stride, const double *params,
                    const double *ts, orc_vf_cb cb, void *cb_ctx, double *ys_out,
                    double *ts_out, int32_t *result, int32_t *stats, double *dense_ts,
                    double *dense_info, int32_t *dense_n, int32_t *event_index,
                    const double *state_in, double *state_out, int nthreads) {
  validate_desc(d);
  if (d->dim > 64 || d->dim < 1) return -1;
  if (d->save_steps < 0) return -1;
  if ((dense_ts != NULL) != (d->save_dense != 0)) return -1;
  if (d->n_event < 0 || d->n_event > ORC_MAX_EVENTS) return -1;
  if (d->levy_area != 0 && d->levy_area != 1) return -1;
  /* the SRKs take the SpaceTimeLevyArea of an SDE's tree (srk.py:374-379) */
  if (ORC_IS_SRK(d->solver) && (d->diffusion == ORC_DIFF_NONE || !d->levy_area)) return -1;
  /* pid.py:437-447: adaptive steps need an error estimate */
  if (d->controller == ORC_PID && d->solver == ORC_SEA) return -1;
  if ((state_in || state_out) && (d->n_step_ts || d->n_jump_ts)) return -2;
  SolveIO io = {d, t0, t1, dt0, time_stride, y0, args, args_stride, params, ts,
                cb, cb_ctx, ys_out, ts_out, result, stats, dense_ts, dense_info, dense_n,
                event_index, state_in, state_out};
#ifdef _OPENMP
  if (nthreads > 0 && d->field != ORC_CALLBACK) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int64_t b = 0; b < B; b++) solve_one(&io, b, NULL);
    return 0;
  }
#endif
  (void)nthreads;
  for (int64_t b = 0; b < B; b++) solve_one(&io, b, NULL);
  return 0;
}

int orc_solve(const orc_desc *d, int64_t B, const double *t0, const double *t1,
              const double *dt0, int64_t time_stride, const double *y0,
              const double *args, int64_t args_stride, const double *params,
              const double *ts, orc_vf_cb cb, void *cb_ctx, double *ys_out,
              double *ts_out, int32_t *result, int32_t *stats, int nthreads) {
  if (d->save_dense) return -1;
  return orc_solve_dense(d, B, t0, t1, dt0, time_stride, y0, args, args_stride, params,
                         ts, cb, cb_ctx, ys_out, ts_out, result, stats, NULL, NULL, NULL,
                         NULL, nthreads);
}

/* ------------------------------------------------------------------------ */
/* DenseInterpolation.evaluate / derivative (_global_interpolation.py:315-393) */
/* over the dense outputs of orc_solve_dense.                                 */
/* ------------------------------------------------------------------------ */
/* d/dtheta of the interp_linear_coeffs coefficients. */
static void interp_deriv_coeffs(int solver, int s, double t, double *ay0, double *ay1,
                                double g[ORC_MAX_S]) {
  for (int j = 0; j < ORC_MAX_S; j++) g[j] = 0.0;
  double t2 = t * t, t3 = t2 * t;
  switch (solver) {
    case ORC_DOPRI8:
      *ay0 = 0.0; *ay1 = 0.0;
      dopri8_weights(t, g, 1);
      break;
    case ORC_TSIT5: {
      /* product rule on the factored weights of tsit5_weights */
      double q, dq;
      *ay0 = 0.0; *ay1 = 0.0;
      q = t2 - 1.4364028541716351 * t + 0.7139816917074209; dq = 2 * t - 1.4364028541716351;
      g[0] = -1.0530884977290216 * ((t - 1.3299890189751412) * q + t * q +
                                     t * (t - 1.3299890189751412) * dq);
      q = t2 - 2.1966568338249754 * t + 1.2949852507374631; dq = 2 * t - 2.1966568338249754;
      g[1] = 0.1017 * (2 * t * q + t2 * dq);
      q = t2 - 2.38535645472061657 * t + 1.57803468208092486; dq = 2 * t - 2.38535645472061657;
      g[2] = 2.490627285651252793 * (2 * t * q + t2 * dq);
      {
        static const double C[4] = {-16.54810288924490272, 47.37952196281928122,
                                    -34.87065786149660974, 2.5};
        static const double A[4] = {1.21712927295533244, 1.203071208372362603, 1.2, 1.0};
        static const double Bq[4] = {0.61620406037800089, 0.658047292653547382,
                                     0.666666666666666667, 0.6};
        for (int m = 0; m < 4; m++) {
          double u = t - A[m], v = t - Bq[m];
          g[3 + m] = C[m] * (v * t2 + u * t2 + u * v * 2 * t);
        }
      }
      break;
    }
    case ORC_DOPRI5: {
      double M = 64 * t3 - 96 * t2 + 32 * t;
      *ay0 = -32 * t3 + 54 * t2 - 22 * t + M;
      *ay1 = -32 * t3 + 42 * t2 - 10 * t;
      for (int j = 0; j < 7; j++) g[j] = M * DOPRI5_CMID[j];
      g[0] += -8 * t3 + 15 * t2 - 8 * t + 1;
      g[6] += 8 * t3 - 9 * t2 + 2 * t;
      break;
    }
    case ORC_HEUN:
      *ay0 = 6 * t2 - 6 * t;
      *ay1 = -6 * t2 + 6 * t;
      g[0] = 3 * t2 - 4 * t + 1;
      g[s - 1] = 3 * t2 - 2 * t;
      break;
    default:
      *ay0 = -1.0; *ay1 = 1.0;
      break;
  }
}

/* searchsorted(ts, t, side) over the whole buffer (unused entries are +inf). */
static int64_t search_sorted(const double *ts, int64_t n, double t, int left) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    int go_right = left ? (ts[mid] < t) : (ts[mid] <= t);
    if (go_right) lo = mid + 1; else hi = mid;
  }
  return lo;
}

int orc_dense_evaluate(const orc_desc *d, int64_t B, const double *t0, const double *t1,
                       int64_t time_stride, const double *y0, const double *dense_ts,
                       const double *dense_info, const int32_t *dense_n, int64_t Q,
                       const double *q, int64_t q_stride, int left, int order,
                       double *out) {
  validate_desc(d);
  const Tableau *tab = tableau_of(d->solver);
  const int D = d->dim, s = tab->s, drec = dense_rec_of(d);
  const int64_t L = d->max_steps + 1;
  for (int64_t b = 0; b < B; b++) {
    const double a0 = t0[b * time_stride], a1 = t1[b * time_stride];
    const int dir = (a0 < a1) ? 1 : -1;
    const double *ts = dense_ts + b * L;
    const int64_t size = dense_n[b];
    for (int64_t m = 0; m < Q; m++) {
      double *o = out + (b * Q + m) * D;
      const double t = q[b * q_stride + m] * dir;
      /* trivial solve: y0 at t0 (_global_interpolation.py:344-345); the
       * derivative of the constant there is zero */
      if (size == 1 && t == a0 * dir) {
        for (int n = 0; n < D; n++) o[n] = order ? 0.0 : y0[b * D + n];
        continue;
      }
      if (size <= 1 || t < ts[0] || t > ts[size - 1]) {  /* _nan_if_out_of_bounds */
        for (int n = 0; n < D; n++) o[n] = NAN;
        continue;
      }
      int64_t idx = search_sorted(ts, L, t, left) - 1; /* _interpret_t */
      if (idx < 0) idx = 0;
      if (idx > size - 2) idx = size - 2;
      const double *r = dense_info + (b * (L - 1) + idx) * drec;
      StepOut so;
      so.dim = D;
      so.tprev = ts[idx];
      so.tnext = ts[idx + 1];
      memcpy(so.y0, r, sizeof(double) * D);
      memcpy(so.y1, r + D, sizeof(double) * D);
      for (int j = 0; j < s; j++) memcpy(so.k[j], r + (2 + j) * D, sizeof(double) * D);
      for (int j = s; j < ORC_MAX_S; j++) memset(so.k[j], 0, sizeof(double) * D);
      if (!order) {
        interp_eval(d->solver, &so, s, t, o);
      } else {
        /* d/dt = (d/dtheta) / (t1 - t0), back in the caller's direction */
        double th = linear_rescale(so.tprev, t, so.tnext), ay0, ay1, g[ORC_MAX_S];
        interp_deriv_coeffs(d->solver, s, th, &ay0, &ay1, g);
        const double span = so.tnext - so.tprev;
        for (int n = 0; n < D; n++) {
          double v = ay0 * so.y0[n] + ay1 * so.y1[n];
          for (int j = 0; j < s; j++) v += g[j] * so.k[j][n];
          o[n] = span == 0.0 ? 0.0 : dir * v / span;
        }
      }
    }
  }
  return 0;
}

/* The ClipStepSizeController helpers on their own (clip.py:55-118, 330-389),
 * for known-answer checks: _find_idx_with_hint, and adapt_step_size after the
 * inner controller proposed (next_t0, next_t1); idx = {step_index, jump_index}. */
int orc_clip_find(const double *ts, int n, int dir, double t, int hint) {
  return clip_find(ts, n, dir, t, hint);
}

int orc_clip_adapt(const double *step_ts, int n_step, const double *jump_ts, int n_jump,
                   int dir, int *idx, double *next_t0, double *next_t1) {
  ClipState c = {step_ts, jump_ts, n_step, n_jump, idx[0], idx[1]};
  int mj = clip_adapt(&c, dir, next_t0, next_t1);
  idx[0] = c.step_index;
  idx[1] = c.jump_index;
  return mj;
}

/* Brownian increments of the oracle's tree, for checking the kernels' tree. */
int orc_vbt_increments(const orc_desc *d, int64_t n, const uint32_t *traj,
                       const double *ta, const double *tb, double *dw) {
  for (int64_t i = 0; i < n; i++) vbt_increment(d, traj[i], ta[i], tb[i], dw + i * d->dim);
  return 0;
}

/* (W, H) increments of the oracle's space-time Levy area tree over [ta, tb]. */
int orc_vbt_levy_increments(const orc_desc *d, int64_t n, const uint32_t *traj,
                            const double *ta, const double *tb, double *dw, double *dh) {
  for (int64_t i = 0; i < n; i++)
    vbt_levy_increment(d, traj[i], ta[i], tb[i], dw + i * d->dim, dh + i * d->dim);
  return 0;
}

/* W(t) and bar H(t) = t H_{0,t} of the Levy area tree on the unit interval. */
int orc_vbt_levy_points(const orc_desc *d, int64_t n, const uint32_t *traj,
                        const double *r, double *w, double *bhh) {
  double tol_unit = d->vbt_tol / (d->vbt_t1 - d->vbt_t0);
  for (int64_t i = 0; i < n; i++)
    vbt_levy_eval_unit(d->seed, traj[i], tol_unit, r[i], d->dim, w + i * d->dim,
                       bhh + i * d->dim);
  return 0;
}

int orc_normal4(uint64_t seed, uint32_t traj, uint32_t node, uint32_t kind, uint32_t q,
                double *z) {
  normal4(seed, traj, node, kind, q, z);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* RecursiveCheckpointAdjoint gradient (_adjoint.py:179-312).                */
/*                                                                           */
/* The reference differentiates the discrete solver: rejected steps get zero */
/* cotangent through `where(keep, ...)` (_integrate.py:422-424) and the step */
/* sizes are under stop_gradient, so the gradient is the VJP of the chain of */
/* accepted steps on the realised time grid.  Checkpointing only changes the */
/* recomputation schedule, not the values, so the oracle tapes every step.   */
/* ------------------------------------------------------------------------ */
static void step_vjp(const Field *F, const Tableau *tab, int dir, const StepOut *so,
                     const double *gy1_in, double kbar[ORC_MAX_S][64], double *gy0,
                     double *gargs, double *gP) {
  const orc_desc *d = F->d;
  const int D = d->dim;
  const double control = dir * (so->tnext - so->tprev);
  double gy1[64];
  memcpy(gy1, gy1_in, sizeof(double) * D);
  double ybar[ORC_MAX_S][64];
  memset(ybar, 0, sizeof ybar);
  if (tab->ssal) {
    for (int n = 0; n < D; n++) ybar[tab->s - 1][n] += gy1[n];
  } else {
    for (int n = 0; n < D; n++) {
      gy0[n] += gy1[n];
      for (int j = 0; j < tab->s; j++) kbar[j][n] += tab->b[j] * gy1[n];
    }
  }
  for (int i = tab->s - 1; i >= 0; i--) {
    double g[64];
    for (int n = 0; n < D; n++) g[n] = kbar[i][n] * control;
    double gyi[64];
    memcpy(gyi, ybar[i], sizeof(double) * D);
    field_drift_vjp(F, so->ystage[i], g, gyi, gargs, gP);
    if (d->diffusion != ORC_DIFF_NONE)
      field_diffusion_vjp(F, so->ystage[i], so->dw, kbar[i], gyi, gargs, gP);
    for (int n = 0; n < D; n++) gy0[n] += gyi[n];
    for (int j = 0; j < i; j++)
      for (int n = 0; n < D; n++) kbar[j][n] += tab->a[i][j] * gyi[n];
  }
}

/* grad_ys: cotangent of the saved ys [B, n_save, D].  Outputs: grad_y0 [B, D],
 * grad_args [B, n_args] (per trajectory), grad_params [n_params] summed over
 * the batch (the caller gives nthreads private buffers via grad_params_tmp). */
int orc_grad_recursive(const orc_desc *d, int64_t B, const double *t0,
                       const double *t1, const double *dt0, int64_t time_stride,
                       const double *y0, const double *args, int64_t args_stride,
                       const double *params, int64_t n_params, const double *ts,
                       const double *grad_ys, double *ys_out, double *ts_out,
                       int32_t *result, int32_t *stats, double *grad_y0,
                       double *grad_args, double *grad_params, int nthreads) {
  validate_desc(d);
  if (d->dim > 64 || d->dim < 1) return -1;
  if (d->save_steps || d->save_dense || d->n_step_ts || d->n_jump_ts || d->n_event)
    return -2; /* forward outputs only */
  if (d->levy_area || ORC_IS_SRK(d->solver)) return -2;
  const Tableau *tab = tableau_of(d->solver);
  const int D = d->dim;
  const int n_save = n_save_of(d);
  SolveIO io = {d, t0, t1, dt0, time_stride, y0, args, args_stride, params, ts,
                NULL, NULL, ys_out, ts_out, result, stats};
  int nt = 1;
#ifdef _OPENMP
  nt = nthreads > 0 ? nthreads : 1;
#endif
  double *gp_all = (double *)calloc((size_t)nt * (size_t)(n_params > 0 ? n_params : 1), sizeof(double));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
#endif
  for (int64_t b = 0; b < B; b++) {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double *gP = n_params > 0 ? gp_all + (size_t)tid * n_params : NULL;
    Tape tape;
    memset(&tape, 0, sizeof tape);
    solve_one(&io, b, &tape);
    Field F = {d, args + b * args_stride, params, NULL, NULL};
    const double *gys = grad_ys + b * (int64_t)n_save * D;
    double gy[64];
    memset(gy, 0, sizeof gy);
    double *gargs = grad_args ? grad_args + b * d->n_args : NULL;
    if (gargs) memset(gargs, 0, sizeof(double) * d->n_args);
    /* t1 save reads the final state; t0 == t1 saves read y0 */
    if (d->save_t1) for (int n = 0; n < D; n++) gy[n] += gys[(int64_t)tape.t1_slot * D + n];
    if (tape.t0_eq_t1) {
      int base = d->save_t0 ? 1 : 0;
      for (int i = 0; i < d->n_ts; i++)
        for (int n = 0; n < D; n++) gy[n] += gys[(int64_t)(base + i) * D + n];
    }
    StepOut so;
    double f0dummy[64];
    double dw[64];
    for (int si = tape.n - 1; si >= 0; si--) {
      TapeStep *st = &tape.steps[si];
      const double *ystart = tape.ys + (int64_t)si * D;
      const double *dwp = NULL;
      if (d->diffusion != ORC_DIFF_NONE) {
        vbt_increment(d, (uint32_t)b, tape.dir * st->tprev, tape.dir * st->tnext, dw);
        dwp = dw;
      }
      rk_step(&F, tab, tape.dir, st->tprev, st->tnext, ystart, 0, f0dummy, dwp, &so);
      double kbar[ORC_MAX_S][64];
      memset(kbar, 0, sizeof kbar);
      double gy0[64], gy1[64];
      memset(gy0, 0, sizeof gy0);
      memcpy(gy1, gy, sizeof(double) * D);
      for (int m = st->save_lo; m < st->save_hi; m++) {
        double tsv = ts_out[b * n_save + m] * tape.dir;
        double th = linear_rescale(st->tprev, tsv, st->tnext);
        double ay0, ay1, g[ORC_MAX_S];
        interp_linear_coeffs(d->solver, tab->s, th, &ay0, &ay1, g);
        const double *go = gys + (int64_t)m * D;
        for (int n = 0; n < D; n++) {
          gy0[n] += ay0 * go[n];
          gy1[n] += ay1 * go[n];
          for (int j = 0; j < tab->s; j++) kbar[j][n] += g[j] * go[n];
        }
      }
      step_vjp(&F, tab, tape.dir, &so, gy1, kbar, gy0, gargs, gP);
      memcpy(gy, gy0, sizeof(double) * D);
    }
    if (d->save_t0) for (int n = 0; n < D; n++) gy[n] += gys[n];
    memcpy(grad_y0 + b * D, gy, sizeof(double) * D);
    free(tape.steps);
    free(tape.ys);
  }
  if (grad_params && n_params > 0) {
    for (int64_t p = 0; p < n_params; p++) {
      double acc = 0.0;
      for (int t = 0; t < nt; t++) acc += gp_all[(size_t)t * n_params + p];
      grad_params[p] = acc;
    }
  }
  free(gp_all);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* BacksolveAdjoint backward (_adjoint.py:572-734).                          */
/*                                                                           */
/* For each pair of adjacent saved times, in reverse, a diffeqsolve of the   */
/* augmented state z = [y | a_y | a_args | a_theta] from ts[j] back to       */
/* ts[j-1] (t0 for the last segment unless t0 itself was saved), started at  */
/* the saved y with a_y += dL/dys[j] (:646-650).  The augmented field is     */
/* AdjointTerm.vf (_term.py:886-910): (f, -a^T df/dy, -a^T df/dargs,          */
/* -a^T df/dtheta).  Solver and controller state carry across segments       */
/* (:656-674); made_jump=True (and the first segment's solver init) means    */
/* the FSAL vector is recomputed at every segment start.  The initial step   */
/* of every segment is chosen as in diffeqsolve with controller_state given  */
/* (_integrate.py:1252-1265): dt0=None -> PID init (0.01 for wrapped terms,   */
/* clipped to dtmin/dtmax); an explicit dt0 -> t0 + dt0 unclipped after the   */
/* first segment.  ConstantStepSize's carried state (constant.py:59-104)     */
/* keeps extending the first segment's grid in later segments, as it does in */
/* the reference.                                                            */
/* ------------------------------------------------------------------------ */
typedef struct {
  int64_t N;       /* augmented size 2D + n_args + n_params */
  /* fsal: f at the current state (the solver state); fsal_new: f at the
   * step's proposed state, committed to fsal only when the step is kept
   * (_integrate.py:424 keeps the solver state of a rejected step) */
  double *k[ORC_MAX_S], *zs, *z1, *err, *fsal, *fsal_new, *f, *sc;
} AugWork;

static void aug_alloc(AugWork *w, int64_t N) {
  w->N = N;
  for (int i = 0; i < ORC_MAX_S; i++) w->k[i] = (double *)calloc((size_t)N, sizeof(double));
  w->zs = (double *)calloc((size_t)N, sizeof(double));
  w->z1 = (double *)calloc((size_t)N, sizeof(double));
  w->err = (double *)calloc((size_t)N, sizeof(double));
  w->fsal = (double *)calloc((size_t)N, sizeof(double));
  w->fsal_new = (double *)calloc((size_t)N, sizeof(double));
  w->f = (double *)calloc((size_t)N, sizeof(double));
  w->sc = (double *)calloc((size_t)N, sizeof(double));
}

static void aug_free(AugWork *w) {
  for (int i = 0; i < ORC_MAX_S; i++) free(w->k[i]);
  free(w->zs); free(w->z1); free(w->err); free(w->fsal); free(w->fsal_new); free(w->f);
  free(w->sc);
}

/* AdjointTerm.vf at z (only the y and a_y parts of z enter). */
static void aug_vf(const Field *F, double t, const double *z, double *out, int64_t N) {
  const orc_desc *d = F->d;
  const int D = d->dim, na = d->n_args;
  field_drift(F, t, z, out);
  memset(out + D, 0, sizeof(double) * (size_t)(N - D));
  field_drift_vjp(F, z, z + D, out + D, na ? out + 2 * D : NULL,
                  N > 2 * D + na ? out + 2 * D + na : NULL);
  for (int64_t n = D; n < N; n++) out[n] = -out[n];
}

/* One explicit RK step of the augmented system (runge_kutta.py:446-1203). */
static void aug_step(const Field *F, const Tableau *tab, int dir, double tprev,
                     double tnext, const double *z0, int have_f0, AugWork *w) {
  const int D2 = 2 * F->d->dim;
  const int64_t N = w->N;
  const double dt = tnext - tprev, control = dir * dt;
  for (int i = 0; i < tab->s; i++) {
    /* stage input: only y and a_y feed the field */
    for (int n = 0; n < D2; n++) {
      double inc = 0.0;
      for (int j = 0; j < i; j++) inc += tab->a[i][j] * w->k[j][n];
      w->zs[n] = z0[n] + inc;
    }
    double ti = (tab->c[i] == 1.0) ? tnext : tprev + tab->c[i] * dt;
    if (i == 0 && have_f0 && tab->fsal) {
      memcpy(w->f, w->fsal, sizeof(double) * (size_t)N);
    } else {
      aug_vf(F, dir * ti, w->zs, w->f, N);
    }
    if (tab->fsal && i == tab->s - 1) memcpy(w->fsal_new, w->f, sizeof(double) * (size_t)N);
    for (int64_t n = 0; n < N; n++) w->k[i][n] = w->f[n] * control;
  }
  for (int64_t n = 0; n < N; n++) {
    if (tab->ssal && n < D2) {
      w->z1[n] = w->zs[n];
    } else {
      double inc = 0.0;
      for (int j = 0; j < tab->s; j++) inc += tab->b[j] * w->k[j][n];
      w->z1[n] = z0[n] + inc;
    }
    double e = 0.0;
    for (int j = 0; j < tab->s; j++) e += tab->e[j] * w->k[j][n];
    w->err[n] = isnan(e) ? INFINITY : e; /* _integrate.py:386 */
  }
}

/* Leaves of the augmented pytree, for the per-leaf NaN rule of pid.py:
 * 475-481: y, a_y, a_args, then each parameter array of the field. */
static int aug_leaves(const orc_desc *d, int64_t *bounds) {
  int nl = 0;
  int64_t o = 0;
  bounds[nl++] = o; o += d->dim;
  bounds[nl++] = o; o += d->dim;
  if (d->n_args) { bounds[nl++] = o; o += d->n_args; }
  if (d->field == ORC_MLP) {
    for (int l = 0; l < d->mlp_depth; l++) {
      int ni = d->mlp_widths[l], no = d->mlp_widths[l + 1];
      bounds[nl++] = o; o += (int64_t)ni * no;
      bounds[nl++] = o; o += no;
    }
  } else if (d->field == ORC_LINEAR) {
    bounds[nl++] = o; o += (int64_t)d->dim * d->dim;
  }
  bounds[nl] = o;
  return nl;
}

typedef struct {
  const orc_desc *d;
  const double *t0, *t1, *dt0;
  int64_t time_stride;
  const double *ts_saved, *ys, *grad_ys;
  const double *args;
  int64_t args_stride;
  const double *params;
  int64_t n_params;
  double *grad_y0, *grad_args;
  int32_t *result, *stats;
} BsIO;

static void backsolve_one(const BsIO *io, int64_t b, double *gP, AugWork *w) {
  const orc_desc *d = io->d;
  const Tableau *tab = tableau_of(d->solver);
  const int D = d->dim, na = d->n_args;
  const int64_t N = w->N;
  const int n_save = n_save_of(d);
  Field F = {d, io->args + b * io->args_stride, io->params, NULL, NULL};
  const double *T = io->ts_saved + b * n_save;
  const double *Y = io->ys + b * (int64_t)n_save * D;
  const double *G = io->grad_ys + b * (int64_t)n_save * D;
  const double t0 = io->t0[b * io->time_stride], t1 = io->t1[b * io->time_stride];
  const int dir = (t0 < t1) ? -1 : 1; /* every segment runs against the forward */
  const int has_dt0 = io->dt0 != NULL;
  const double h0 = has_dt0 ? fabs(io->dt0[b * io->time_stride]) : 0.0;
  const double eord = error_order_of(d, tab);
  const int n_norm = d->norm == ORC_NORM_ADJOINT_SEMI ? 2 * D : (int)N;
  int64_t leaf[64];
  const int nleaf = aug_leaves(d, leaf);

  double *z = (double *)calloc((size_t)N, sizeof(double));
  CtrlState cs;
  memset(&cs, 0, sizeof cs);
  int first_seg = 1, result = ORC_SUCCESSFUL;
  int tot = 0, acc = 0, rej = 0;
  const int jlo = d->save_t0 ? 1 : 0;
  for (int j = n_save - 1; j >= jlo; j--) {
    const double target = j >= 1 ? T[j - 1] : t0;
    memcpy(z, Y + (int64_t)j * D, sizeof(double) * D);
    for (int n = 0; n < D; n++) z[D + n] += G[(int64_t)j * D + n];
    const double ts_ = dir * T[j], te = dir * target;
    double tnext;
    if (d->controller == ORC_PID) {
      if (first_seg || !has_dt0) {
        double h = has_dt0 ? h0 : 0.01;
        if (!isnan(d->dtmax)) h = h < d->dtmax ? h : d->dtmax;
        if (!isnan(d->dtmin)) h = h > d->dtmin ? h : d->dtmin;
        tnext = ts_ + h;
      } else {
        tnext = ts_ + h0;
      }
      if (first_seg) { cs.prev_inv = 1.0; cs.prev_prev_inv = 1.0; cs.at_dtmin = 0; }
    } else {
      if (first_seg) {
        cs.steps_completed = 1;
        cs.num_steps = (int)ceil((te - ts_) / nextafter(h0, INFINITY));
        cs.t0_sim = ts_; cs.t1_sim = te;
      }
      tnext = ts_ + h0;
    }
    first_seg = 0;
    tnext = tnext < te ? tnext : te;
    double tprev = ts_;
    double floor_te = te;
    for (int i = 0; i < 100; i++) floor_te = prevbefore(floor_te);
    int have_f0 = 0, nsteps = 0, seg_result = ORC_SUCCESSFUL;
    while (tprev < te && seg_result == ORC_SUCCESSFUL) {
      if (nsteps >= d->max_steps) break;
      aug_step(&F, tab, dir, tprev, tnext, z, have_f0, w);
      int keep, cres = ORC_SUCCESSFUL;
      double nt0, nt1;
      if (d->controller == ORC_PID) {
        double ssum = 0.0;
        for (int l = 0; l < nleaf; l++) {
          if (leaf[l] >= n_norm) break;
          int any_nan = 0;
          for (int64_t n = leaf[l]; n < leaf[l + 1]; n++) any_nan |= isnan(w->z1[n]);
          for (int64_t n = leaf[l]; n < leaf[l + 1] && n < n_norm; n++) {
            double a0 = fabs(z[n]), a1 = fabs(any_nan ? z[n] : w->z1[n]);
            double ym = a0 > a1 ? a0 : a1;
            double s = w->err[n] / (d->atol + ym * d->rtol);
            ssum += s * s;
          }
        }
        double scaled = sqrt(ssum) / sqrt((double)n_norm);
        keep = pid_adapt(d, eord, tprev, tnext, scaled, &cs, &nt0, &nt1, &cres);
      } else {
        keep = constant_adapt(tnext, &cs, &nt0, &nt1);
      }
      nt0 = nt0 < te ? nt0 : te;
      if (nt1 > floor_te) nt1 = keep ? te : nt0 + 0.5 * (te - nt0);
      if (keep) {
        memcpy(z, w->z1, sizeof(double) * (size_t)N);
        if (tab->fsal) {
          memcpy(w->fsal, w->fsal_new, sizeof(double) * (size_t)N);
          have_f0 = 1;
        }
      }
      if (seg_result == ORC_SUCCESSFUL) seg_result = cres;
      nsteps++;
      tot++;
      if (keep) acc++; else rej++;
      tprev = nt0;
      tnext = nt1;
    }
    if (seg_result == ORC_SUCCESSFUL && tprev < te) seg_result = ORC_MAX_STEPS_REACHED;
    if (result == ORC_SUCCESSFUL) result = seg_result;
  }
  if (d->save_t0)
    for (int n = 0; n < D; n++) z[D + n] += G[n];
  memcpy(io->grad_y0 + b * D, z + D, sizeof(double) * D);
  if (io->grad_args && na) memcpy(io->grad_args + b * na, z + 2 * D, sizeof(double) * na);
  if (gP)
    for (int64_t p = 0; p < io->n_params; p++) gP[p] += z[2 * D + na + p];
  io->result[b] = result;
  io->stats[b * 3 + 0] = tot;
  io->stats[b * 3 + 1] = acc;
  io->stats[b * 3 + 2] = rej;
  free(z);
}

/* ts_saved [B, n_save] and ys [B, n_save, D] are the forward's saved outputs,
 * grad_ys their cotangent.  d describes the backward solve (its solver,
 * controller and norm) and the forward's SaveAt.  Outputs: grad_y0 [B, D],
 * grad_args [B, n_args], grad_params [n_params] summed over the batch,
 * result [B] and stats [B, 3] (steps, accepted, rejected over all segments). */
int orc_backsolve(const orc_desc *d, int64_t B, const double *t0, const double *t1,
                  const double *dt0, int64_t time_stride, const double *ts_saved,
                  const double *ys, const double *grad_ys, const double *args,
                  int64_t args_stride, const double *params, int64_t n_params,
                  double *grad_y0, double *grad_args, double *grad_params,
                  int32_t *result, int32_t *stats, int nthreads) {
  validate_desc(d);
  if (d->dim > 64 || d->dim < 1) return -1;
  if (d->field == ORC_CALLBACK || d->diffusion != ORC_DIFF_NONE) return -2;
  if (d->save_steps || d->save_dense || d->n_step_ts || d->n_jump_ts || d->n_event) return -2;
  if (d->levy_area || ORC_IS_SRK(d->solver)) return -2;
  const int64_t N = 2 * (int64_t)d->dim + d->n_args + n_params;
  BsIO io = {d, t0, t1, dt0, time_stride, ts_saved, ys, grad_ys, args, args_stride,
             params, n_params, grad_y0, grad_args, result, stats};
  int nt = 1;
#ifdef _OPENMP
  nt = nthreads > 0 ? nthreads : 1;
#endif
  (void)nthreads;
  double *gp_all = (double *)calloc((size_t)nt * (size_t)(n_params > 0 ? n_params : 1), sizeof(double));
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    AugWork w;
    aug_alloc(&w, N);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for (int64_t b = 0; b < B; b++)
      backsolve_one(&io, b, n_params > 0 ? gp_all + (size_t)tid * n_params : NULL, &w);
    aug_free(&w);
  }
  if (grad_params && n_params > 0) {
    for (int64_t p = 0; p < n_params; p++) {
      double acc = 0.0;
      for (int t = 0; t < nt; t++) acc += gp_all[(size_t)t * n_params + p];
      grad_params[p] = acc;
    }
  }
  free(gp_all);
  return 0;
}

int orc_abi_version(void) { return 1; }
int orc_desc_size(void) { return (int)sizeof(orc_desc); }

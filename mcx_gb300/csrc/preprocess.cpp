// preprocess.cpp -- host-side Config preparation for callers that do not link MCX's own
// front-end code (mcx_utils.c).
//
// The MCX front-ends run mcx_initcfg / mcx_validatecfg / mcx_preprocess / mcx_maskdet before
// they call mcx_run_simulation; the engine receives an already prepared Config.  The pmcx-style
// Python API of this package (mcx_gb300.run) has no mcx_utils.c to call, so the subset of that
// preparation which the transport path depends on is restated here:
//   mcxg_initcfg      <- mcx_initcfg        src/mcx_utils.c:248-378   (default values)
//   mcxg_validatecfg  <- mcx_validatecfg    src/mcx_utils.c:3748-3857 (origin shift, time gates)
//                        mcx_preprocess     src/mcx_utils.c:1525-1820 (direction, media, launch voxel)
//   mcxg_maskdet      <- mcx_maskdet        src/mcx_utils.c:4214-4340 (label-media branch)
//                        mcx_prep_polarized src/mcx_utils.c:1831-1871 (Mie tables), with the Mie
//                        series of src/mcx_mie.cpp:91-216 restated
// Out of this restatement (and rejected by the engine): seed files, extra sources, shapes/JSON
// parsing.

#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <algorithm>
#include <thread>
#include <vector>

#include "../../include/mcx_abi.h"
#include "../../include/mcx_gb300.h"
#include "mcxg_common.h"
#include "transport.cuh"

using namespace mcxg;

namespace {

const char kBoundaryCond[] = {'_', 'r', 'a', 'm', 'c', '\0'};
const char kBoundaryDet[] = {'0', '1', '\0'};

// Replace a boundary character by its index in `table` (src/mcx_utils.c:5428-5441).
bool lookup_index(char* key, const char* table) {
    for (int i = 0; table[i]; i++) {
        if (std::tolower((unsigned char)*key) == table[i]) {
            *key = (char)i;
            return true;
        }
    }
    return false;
}

}  // namespace

extern "C" void mcxg_initcfg(Config* cfg) {
    std::memset(cfg, 0, sizeof(Config));
    cfg->mediabyte = 1;
    cfg->steps.x = cfg->steps.y = cfg->steps.z = 1.f;
    cfg->nblocksize = 64;
    cfg->nthread = 1 << 14;
    cfg->isreflect = 1;
    cfg->isref3 = 1;
    cfg->isnormalized = 1;
    cfg->issavedet = 1;
    cfg->respin = 1;
    cfg->issave2pt = 1;
    cfg->flog = stdout;
    cfg->sradius = -2.f;
    cfg->tstep = 1.f / FLT_EPSILON;
    cfg->unitinmm = 1.f;
    cfg->maxdetphoton = 1000000;
    cfg->maxjumpdebug = 10000000;
    cfg->autopilot = 1;
    cfg->seed = 0x623F9A9E;
    std::memcpy(cfg->his.magic, "MCXH", 4);
    cfg->his.version = 1;
    cfg->his.unitinmm = 1.f;
    cfg->his.normalizer = 1.f;
    cfg->his.respin = 1;
    cfg->his.srcnum = 1;
    cfg->savedetflag = 0x5;
    cfg->his.savedetflag = cfg->savedetflag;
    cfg->maxvoidstep = 1000;
    cfg->voidtime = 1;
    cfg->srcnum = 1;
    cfg->outputtype = otFlux;
    cfg->outputformat = 5;           // jnii
    cfg->srcpos.w = 1.f;
    cfg->gscatter = 1000000000u;
    cfg->his.totalsource = 1;
    cfg->deviceid[0] = '1';
    cfg->parentid = mpPython;
}

// Mark every voxel that touches a detector sphere on an interface or on the bounding box by
// setting bit 31 (label-media branch of src/mcx_utils.c:4214-4340).
extern "C" void mcxg_maskdet(Config* cfg) {
    const uint32_t dx = cfg->dim.x + 2, dy = cfg->dim.y + 2, dz = cfg->dim.z + 2;
    const int isonecube = (cfg->dim.x == 1) && (cfg->dim.y == 1) && (cfg->dim.z == 1);
    static const float corners[8][3] = {{0.f, 0.f, 0.f}, {1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f},
                                        {1.f, 1.f, 0.f}, {1.f, 0.f, 1.f}, {0.f, 1.f, 1.f}, {1.f, 1.f, 1.f}};
    // pad with one layer of zeros so neighbour tests never leave the array
    std::vector<uint32_t> pad((size_t)dx * dy * dz, 0u);
    for (uint32_t z = 1; z <= cfg->dim.z; z++)
        for (uint32_t y = 1; y <= cfg->dim.y; y++)
            std::memcpy(&pad[(size_t)z * dy * dx + (size_t)y * dx + 1],
                        cfg->vol + (size_t)(z - 1) * cfg->dim.y * cfg->dim.x + (size_t)(y - 1) * cfg->dim.x,
                        cfg->dim.x * sizeof(uint32_t));
    const long sx = 1, sy = (long)dx, sz = (long)dx * dy;
    for (uint32_t d = 0; d < cfg->detnum; d++) {
        const float4 dp = cfg->detpos[d];
        const float radius = std::fabs(dp.w);
        const float d2max = (radius + 1.7321f) * (radius + 1.7321f);
        for (float z = -radius - 1.f; z <= radius + 1.f; z += 0.5f) {
            const float iz = z + dp.z;
            for (float y = -radius - 1.f; y <= radius + 1.f; y += 0.5f) {
                const float iy = y + dp.y;
                for (float x = -radius - 1.f; x <= radius + 1.f; x += 0.5f) {
                    const float ix = x + dp.x;
                    if (iz < 0 || ix < 0 || iy < 0 || ix >= cfg->dim.x || iy >= cfg->dim.y || iz >= cfg->dim.z ||
                        x * x + y * y + z * z > (radius + 1.f) * (radius + 1.f))
                        continue;
                    float mind2 = 1.f / FLT_EPSILON;
                    for (int c = 0; c < 8; c++) {
                        const float rx = (int)ix - dp.x + corners[c][0];
                        const float ry = (int)iy - dp.y + corners[c][1];
                        const float rz = (int)iz - dp.z + corners[c][2];
                        const float d2 = rx * rx + ry * ry + rz * rz;
                        if (d2 > d2max) { mind2 = 1.f / FLT_EPSILON; break; }
                        if (d2 < mind2) mind2 = d2;
                    }
                    const float lim = radius + 0.5f * (1.f + isonecube);
                    if (mind2 == 1.f / FLT_EPSILON || mind2 >= lim * lim) continue;
                    const long id = (long)((int)(iz + 1.f)) * sz + (long)((int)(iy + 1.f)) * sy + (int)(ix + 1.f);
                    if (!pad[id]) continue;
                    // interior voxel: all 26 neighbours non-zero -> not on an interface
                    bool interior = true;
                    for (int oz = -1; oz <= 1 && interior; oz++)
                        for (int oy = -1; oy <= 1 && interior; oy++)
                            for (int ox = -1; ox <= 1; ox++) {
                                if (!ox && !oy && !oz) continue;
                                if (!pad[id + oz * sz + oy * sy + ox * sx]) { interior = false; break; }
                            }
                    if (!interior)
                        cfg->vol[(size_t)((int)iz) * cfg->dim.y * cfg->dim.x + (size_t)((int)iy) * cfg->dim.x + (int)ix] |= kDET_MASK;
                }
            }
        }
    }
}

namespace {

constexpr int kNAngles = 1000;      // NANGLES, src/mcx_const.h:59

typedef std::complex<double> cplx;

void put_mueller(float4& out, cplx s1, cplx s2) {
    const double a1 = std::abs(s1), a2 = std::abs(s2);
    const cplx c = std::conj(s1) * s2;
    out = make_float4((float)(0.5 * a2 * a2 + 0.5 * a1 * a1), (float)(0.5 * a2 * a2 - 0.5 * a1 * a1),
                      (float)std::real(c), (float)std::imag(c));
}

// Small spheres (m x < 0.1): the dipole/quadrupole expansion of Wiscombe (1980) in the form MCX
// evaluates it (src/mcx_mie.cpp:232-312), for a real relative index m.  The coefficients a1, b1
// and a2 follow Wiscombe's series in x^2; S1 = a1 + (b1 + a2) mu and S2 = b1 + (a1 + a2)(2 mu^2 - 1)
// after scaling by 3/2 x^3 (a2 also by 5/3), which is how MCX combines them.
void small_mie(double x, double m, const std::vector<double>& mu, float4* sm, double& qsca, double& g) {
    const double m2 = m * m, m4 = m2 * m2, x2 = x * x, x3 = x2 * x, x4 = x2 * x2;
    const cplx z0(0.0, m2 - 1.0);          // i (m^2 - 1)
    const cplx z1 = 2.0 / 3.0 * z0;
    const cplx z3 = z1 * cplx(1.0 - 0.1 * x2 + (4.0 * m2 + 5.0) * x4 / 1400.0, 0.0);
    const cplx z4 = x3 * (1.0 - 0.1 * x2) * z1;
    const cplx den(2.0 + m2 + (1 - 0.7 * m2) * x2 + (8 * m4 - 385 * m2 + 350.0) / 1400 * x4 + std::real(z4), std::imag(z4));
    cplx a1 = z3 / den;
    cplx b1 = (x2 / 45.0 * z0) * (cplx(1.0 + (2.0 * m2 - 5.0) * x2 / 70.0, 0.0) / cplx(1.0 - (2.0 * m2 - 5.0) * x2 / 30.0, 0.0));
    cplx a2 = ((1.0 - x2 / 14) * x2 / 15.0 * z0) / cplx(2.0 * m2 + 3.0 - (m2 / 7.0 - 0.5) * x2, 0.0);
    const double aa1 = std::abs(a1), ab1 = std::abs(b1), aa2 = std::abs(a2);
    const double t = aa1 * aa1 + ab1 * ab1 + 5.0 / 3.0 * aa2 * aa2;
    qsca = 6.0 * x4 * t;
    g = (std::real(a1) * (std::real(a2) + std::real(b1)) + std::imag(a1) * (std::imag(a2) + std::imag(b1))) / t;
    const double sc = x3 * 1.5;
    a1 *= sc;
    b1 *= sc;
    a2 *= sc * 5.0 / 3.0;
    for (size_t k = 0; k < mu.size(); k++) {
        const double c2 = 2 * mu[k] * mu[k] - 1;
        put_mueller(sm[k], a1 + (b1 + a2) * mu[k], b1 + (a1 + a2) * c2);
    }
}

// Lorenz-Mie scattering by a homogeneous sphere of size parameter x and real relative refractive
// index m, in the series form of Wiscombe (1980) as MCX evaluates it (src/mcx_mie.cpp:91-216):
// the logarithmic derivative D_n(mx) by upward recurrence (MCX fills D_0..D_{nstop-1} and the
// last term of the series sees D_nstop = 0), Riccati-Bessel psi_n and xi_n = psi_n + i chi_n by
// upward recurrence, the coefficients a_n and b_n, the amplitudes S1 and S2 at cos(theta) = mu[k],
// the scattering efficiency and the asymmetry g.  Writes the Mueller elements per angle as
// (S11, S12, S33, S34).
void mie(double x, double m, const std::vector<double>& mu, float4* sm, double& qsca, double& g) {
    if (x <= 0.0) MCXG_RAISE(-6, "sphere size must be positive");
    if (x > 20000.0) MCXG_RAISE(-6, "spheres with x>20000 are not validated");
    if (std::abs(m) * x < 0.1) {
        small_mie(x, m, mu, sm, qsca, g);
        return;
    }
    const int nk = (int)mu.size();
    const long nstop = (long)std::floor(x + 4.05 * std::pow(x, 0.33333) + 2.0);
    std::vector<cplx> s1(nk), s2(nk);
    std::vector<double> pi1(nk, 1.0), pi0(nk, 0.0), tau(nk, 0.0);
    const double z = m * x, zinv = 1.0 / z;
    std::vector<double> D(nstop + 1, 0.0);
    D[0] = 1.0 / std::tan(z);
    for (long k = 1; k < nstop; k++) D[k] = 1.0 / (k * zinv - D[k - 1]) - k * zinv;
    double psi0 = std::sin(x), psi1 = psi0 / x - std::cos(x);
    cplx xi0(psi0, std::cos(x)), xi1(psi1, std::cos(x) / x + std::sin(x));
    cplx anm1(0.0, 0.0), bnm1(0.0, 0.0);
    qsca = 0.0;
    g = 0.0;
    for (long n = 1; n <= nstop; n++) {
        const double da = D[n] / m + n / x, db = D[n] * m + n / x;
        const cplx an = (da * psi1 - psi0) / (da * xi1 - xi0);
        const cplx bn = (db * psi1 - psi0) / (db * xi1 - xi0);
        const double f = (2.0 * n + 1.0) / (n + 1.0) / n;
        for (int k = 0; k < nk; k++) {
            tau[k] = n * mu[k] * pi1[k] - (n + 1) * pi0[k];
            const double al = f * pi1[k], be = f * tau[k];
            s1[k] += cplx(al * an.real() + be * bn.real(), al * an.imag() + be * bn.imag());
            s2[k] += cplx(al * bn.real() + be * an.real(), al * bn.imag() + be * an.imag());
        }
        for (int k = 0; k < nk; k++) {
            const double p = pi1[k];
            pi1[k] = ((2.0 * n + 1.0) * mu[k] * pi1[k] - (n + 1.0) * pi0[k]) / n;
            pi0[k] = p;
        }
        g += (n - 1.0 / n) * (anm1.real() * an.real() + anm1.imag() * an.imag() + bnm1.real() * bn.real() + bnm1.imag() * bn.imag());
        g += (2.0 * n + 1.0) / n / (n + 1.0) * (an.real() * bn.real() + an.imag() * bn.imag());
        const double aa = std::abs(an), ab = std::abs(bn);
        qsca += (2.0 * n + 1.0) * (aa * aa + ab * ab);
        const cplx xi = (2.0 * n + 1.0) / x * xi1 - xi0;
        xi0 = xi1;
        xi1 = xi;
        psi0 = psi1;
        psi1 = xi1.real();
        anm1 = an;
        bnm1 = bn;
    }
    qsca *= 2.0 / (x * x);
    g *= 4.0 / qsca / (x * x);
    for (int k = 0; k < nk; k++) put_mueller(sm[k], s1[k], s2[k]);
}

// mcx_prep_polarized (src/mcx_utils.c:1831-1871): each polarised medium's Mueller table and, from
// its spheres (radius r um, number density rho per um^3, indices nsph in nmed at lambda nm), its
// scattering coefficient; a medium whose prop row already holds mus (and g) gets the density
// that reproduces that mus (or mus(1 - g)).  The angle grid, size parameter and cross-section use
// single-precision pi and float products as MCX does, so the tables agree bit for bit.  The table
// is malloc'ed into cfg->smatrix.
void prep_polarized(Config* cfg) {
    const float pi_f = 3.14159265358979f, two_pi_f = 6.28318530717959f;
    std::vector<double> mu(kNAngles);
    for (int i = 0; i < kNAngles; i++) mu[i] = std::cos((double)(pi_f * (float)i / (float)(kNAngles - 1)));
    std::free(cfg->smatrix);
    cfg->smatrix = (float4*)std::malloc(sizeof(float4) * kNAngles * cfg->polmedianum);
    if (!cfg->smatrix) MCXG_RAISE(-4, "out of host memory for the scattering matrices");
    for (uint32_t i = 0; i < cfg->polmedianum; i++) {
        POLMedium& pm = cfg->polprop[i];
        Medium& md = cfg->prop[i + 1];
        md.mua = pm.mua;
        md.n = pm.nmed;
        const double x = (double)(two_pi_f * pm.r * pm.nmed) / (cfg->lambda * 1e-3);
        const float area = pi_f * pm.r * pm.r;                   // um^2
        double qsca = 0.0, g = 0.0;
        mie(x, (double)(pm.nsph / pm.nmed), mu, cfg->smatrix + (size_t)i * kNAngles, qsca, g);
        if (md.mus > kEPS) {
            float target = md.mus;
            if (md.g < 1.f - kEPS) {
                const float musp = md.mus * (1.f - md.g);
                target = (float)(musp / (1.0 - g));
            }
            pm.rho = (float)(target / qsca / area * 1e-3);
        }
        md.mus = (float)(qsca * area * pm.rho * 1e3);
        md.g = (float)g;
    }
}

// dst[z][y][x] = src[x][y][z] for a d.x x d.y x d.z volume: for each y a (d.x x d.z) matrix
// transpose, done in 32 x 32 tiles so that both sides stay in cache lines, the y slabs shared out
// over a few threads for large volumes.
void row_to_column_major(const uint32_t* src, uint32_t* dst, uint3 d) {
    constexpr uint32_t T = 32;
    auto slab = [&](uint32_t y0, uint32_t y1) {
        for (uint32_t y = y0; y < y1; y++)
            for (uint32_t x0 = 0; x0 < d.x; x0 += T)
                for (uint32_t z0 = 0; z0 < d.z; z0 += T) {
                    const uint32_t x1 = std::min(d.x, x0 + T), z1 = std::min(d.z, z0 + T);
                    for (uint32_t x = x0; x < x1; x++) {
                        const uint32_t* s = src + ((size_t)x * d.y + y) * d.z;
                        for (uint32_t z = z0; z < z1; z++) dst[((size_t)z * d.y + y) * d.x + x] = s[z];
                    }
                }
    };
    const size_t n = (size_t)d.x * d.y * d.z;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = (n < (1u << 20)) ? 1u : std::min<unsigned>({hw, 8u, d.y});
    if (nt <= 1) {
        slab(0, d.y);
        return;
    }
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++)
        th.emplace_back(slab, (uint32_t)((uint64_t)d.y * t / nt), (uint32_t)((uint64_t)d.y * (t + 1) / nt));
    for (auto& t : th) t.join();
}

void validate(Config* cfg) {
    // replay of saved photons (src/mcx_utils.c:1651-1664)
    if (cfg->seed == kSEED_FROM_FILE && (cfg->respin > 1 || cfg->respin < 0)) {
        cfg->respin = 1;
        if (cfg->flog) fprintf(cfg->flog, "WARNING: respin is disabled in the replay mode\n");
    }
    if (cfg->replaydet > (int)cfg->detnum) MCXG_RAISE(-4, "replay detector ID exceeds the maximum detector number");
    if (cfg->replaydet == -1 && cfg->detnum == 1) cfg->replaydet = 1;


    // mcx_validatecfg: grid-origin shift, time gates (src/mcx_utils.c:3761-3795)
    if (!cfg->issrcfrom0) {
        cfg->srcpos.x -= 1.f; cfg->srcpos.y -= 1.f; cfg->srcpos.z -= 1.f;
        for (uint32_t i = 0; cfg->srcdata && i < cfg->extrasrclen; i++) {      // 3766-3771
            cfg->srcdata[i].srcpos.x -= 1.f; cfg->srcdata[i].srcpos.y -= 1.f; cfg->srcdata[i].srcpos.z -= 1.f;
        }
        for (uint32_t i = 0; i < cfg->detnum; i++) {
            cfg->detpos[i].x -= 1.f; cfg->detpos[i].y -= 1.f; cfg->detpos[i].z -= 1.f;
        }
        cfg->issrcfrom0 = 1;   // prevents a second shift if validate runs twice
    }
    if (cfg->tstep == 0.f) cfg->tstep = cfg->tend;
    if (cfg->tstart >= cfg->tend || cfg->tstep == 0.f) MCXG_RAISE(-6, "incorrect time gate settings");
    if (cfg->steps.x == 0.f || cfg->steps.y == 0.f || cfg->steps.z == 0.f) MCXG_RAISE(-6, "field 'steps' can not have zero elements");
    const int gates = (int)((cfg->tend - cfg->tstart) / cfg->tstep + 0.5f);
    if ((int)cfg->maxgate > gates) cfg->maxgate = gates;
    if (cfg->seed < 0 && cfg->seed != kSEED_FROM_FILE) cfg->seed = (int)time(nullptr);

    // mcx_preprocess (src/mcx_utils.c:1525-1820), label-media subset
    double len = std::sqrt((double)cfg->srcdir.x * cfg->srcdir.x + (double)cfg->srcdir.y * cfg->srcdir.y +
                           (double)cfg->srcdir.z * cfg->srcdir.z);
    if (len < FLT_EPSILON) MCXG_RAISE(-4, "source initial direction vector can not have a length of 0");
    const float inv = (float)(1.0 / len);
    cfg->srcdir.x *= inv; cfg->srcdir.y *= inv; cfg->srcdir.z *= inv;
    if (cfg->debuglevel & kDebugMoveOnly) {     // trajectories only (src/mcx_utils.c:1539-1542)
        cfg->issave2pt = 0;
        cfg->issavedet = 0;
    }

    int isbcdet = 0;
    for (int i = 0; i < 6; i++)
        if (cfg->bc[i] && !lookup_index(cfg->bc + i, kBoundaryCond)) MCXG_RAISE(-4, "unknown boundary condition specifier");
    for (int i = 6; i < 12; i++) {
        if (cfg->bc[i] && !lookup_index(cfg->bc + i, kBoundaryDet)) MCXG_RAISE(-4, "unknown boundary detection flags");
        if (cfg->bc[i]) isbcdet = 1;
    }
    if (cfg->medianum == 0) MCXG_RAISE(-4, "you must define the 'prop' field in the input structure");
    if (cfg->dim.x == 0 || cfg->dim.y == 0 || cfg->dim.z == 0) MCXG_RAISE(-4, "the 'vol' field in the input structure can not be empty");
    if (cfg->mediabyte > 4 && !media_words(cfg->mediabyte))
        MCXG_RAISE(-6, "the GB300 engine supports label media (mediabyte 1, 2, 4) and the per-voxel formats 96-104");
    check_source(cfg);

    // polarised media (src/mcx_utils.c:1569-1591): label volumes only, one sphere population per
    // medium after the background, a wavelength, and a Stokes vector of non-negative intensity
    // Stokes vectors in trajectories only for trajectories of polarised runs (src/mcx_utils.c:1549-1552)
    if (!(cfg->debuglevel & (kDebugMove | kDebugMoveOnly)) || !(cfg->mediabyte <= 4 && cfg->polmedianum > 0))
        cfg->istrajstokes = 0;
    if (cfg->polprop && cfg->polmedianum) {
        if (cfg->mediabyte > 4) MCXG_RAISE(-1, "Unsupported media format");
        if (cfg->medianum != cfg->polmedianum + 1) MCXG_RAISE(-6, "number of particle types does not match number of media");
        if (cfg->lambda == 0.f) MCXG_RAISE(-1, "you must specify light wavelength lambda to run polarized photon simulation");
        if (cfg->srciquv.x < 0.f) MCXG_RAISE(-4, "initial total light intensity must not be negative");
        if (cfg->srciquv.y < -1.f || cfg->srciquv.y > 1.f || cfg->srciquv.z < -1.f || cfg->srciquv.z > 1.f ||
            cfg->srciquv.w < -1.f || cfg->srciquv.w > 1.f)
            MCXG_RAISE(-4, "initial Q, U and V must be floating-point numbers between -1 and 1");
        prep_polarized(cfg);
    }

    if (cfg->steps.x != 1.f && cfg->unitinmm == 1.f) cfg->unitinmm = cfg->steps.x;
    if (cfg->unitinmm != 1.f) {
        cfg->steps.x = cfg->steps.y = cfg->steps.z = cfg->unitinmm;
        for (uint32_t i = 1; i < cfg->medianum; i++) {
            cfg->prop[i].mus *= cfg->unitinmm;
            cfg->prop[i].mua *= cfg->unitinmm;
        }
    }
    if (cfg->isrowmajor) {
        // C-order input: transpose to MCX's x-fastest order (src/mcx_utils.c:1620-1631)
        std::vector<uint32_t> tmp((size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z);
        row_to_column_major(cfg->vol, tmp.data(), cfg->dim);
        std::memcpy(cfg->vol, tmp.data(), tmp.size() * sizeof(uint32_t));
        cfg->isrowmajor = 0;
    }
    if (cfg->issavedet && cfg->detnum == 0 && isbcdet == 0) cfg->issavedet = 0;
    if (cfg->issavedet == 0) {
        cfg->issaveexit = 0;
        cfg->ismomentum = 0;
        cfg->savedetflag = 0;
    }
    if (cfg->respin == 0) MCXG_RAISE(-1, "respin number can not be 0, check your -r/--repeat input or cfg.respin value");
    for (uint32_t i = 0; i < cfg->medianum; i++) {
        if (cfg->prop[i].mus == 0.f) {
            cfg->prop[i].mus = FLT_EPSILON;
            cfg->prop[i].g = 1.f;
        }
    }
    if (cfg->srcpos.w == 0.f) cfg->srcpos.w = 1.f;
    const size_t nvox = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
    if (cfg->mediabyte <= 4) {
        uint32_t maxlabel = 0;
        for (size_t i = 0; i < nvox; i++) maxlabel = std::max(maxlabel, cfg->vol[i] & kMED_MASK);
        if (cfg->medianum <= maxlabel) MCXG_RAISE(-4, "input media optical properties are less than the labels in the volume");
    }

    // launch voxel and medium of point sources (src/mcx_utils.c:1737-1760); the other shapes keep
    // srcparam2 as their parameters
    uint32_t idx = 0, med = 0;
    if (src_is_point((unsigned char)cfg->srctype) && !(cfg->srcpos.x < 0.f || cfg->srcpos.y < 0.f || cfg->srcpos.z < 0.f || cfg->srcpos.x >= cfg->dim.x ||
          cfg->srcpos.y >= cfg->dim.y || cfg->srcpos.z >= cfg->dim.z)) {
        idx = (uint32_t)((int)std::floor(cfg->srcpos.z) * (cfg->dim.y * cfg->dim.x) + (int)std::floor(cfg->srcpos.y) * cfg->dim.x +
                         (int)std::floor(cfg->srcpos.x));
        med = cfg->vol[idx] & kMED_MASK;
    }
    if (src_is_point((unsigned char)cfg->srctype)) {
        std::memcpy(&cfg->srcparam2.z, &idx, 4);
        std::memcpy(&cfg->srcparam2.w, &med, 4);
    }

    if (cfg->issavedet) mcxg_maskdet(cfg);
    for (int i = 0; i < MCXG_MAX_DEVICE; i++)
        if (cfg->deviceid[i] == '0') cfg->deviceid[i] = '\0';
    if (cfg->ismomentum) cfg->savedetflag |= 0x8;
    if (cfg->issaveexit) cfg->savedetflag |= 0x30;
    if (cfg->polmedianum)             // src/mcx_utils.c:1788-1795: P, V, W0 and the Stokes vector
        cfg->savedetflag |= 0x4u | 0x20u | 0x40u | 0x80u;
    else
        cfg->savedetflag &= ~0x80u;   // no Stokes vector without polarisation
    if (cfg->issavedet && cfg->savedetflag == 0) cfg->savedetflag = 0x5;
    // per-voxel media have no labels: no per-medium record columns (src/mcx_utils.c:1801-1806)
    // per-voxel formats carry no per-medium slots (src/mcx_utils.c:1801-1803, mediabyte >= 100); for
    // mediabyte 96, 98 and 99 MCX keeps the flags and indexes the slots by the voxel word, past the
    // end of the record, so the engine clears them for every non-label format
    if (cfg->mediabyte > 4 && cfg->savedetflag) cfg->savedetflag &= ~(0x2u | 0x4u | 0x8u | 0x80u);
    // diffuse reflectance (src/mcx_utils.c:3757-3759, 1808-1818): needs the field; mode 2 keeps one
    // detected record per void voxel with the exit weight and the weighted partial paths summed
    // there (saveexitppath, src/mcx_core.cu:272-285)
    if (!cfg->issave2pt) cfg->issaveref = 0;
    if (cfg->issaveref > 1) {          // exit weight and paths per void voxel in the detected buffer
        if (!cfg->issavedet) MCXG_RAISE(-4, "you must have at least two outputs if issaveref is greater than 1");
        const uint32_t nv = cfg->dim.x * cfg->dim.y * cfg->dim.z;
        if (nv > cfg->maxdetphoton) {
            if (cfg->flog) fprintf(cfg->flog, "you must set --maxdetphoton larger than the total size of the voxels when --issaveref is greater than 1; autocorrecting ...\n");
            cfg->maxdetphoton = nv;
        }
        cfg->savedetflag = 0x5;
    }

    // history header bookkeeping done at the end of mcx_validatecfg (src/mcx_utils.c:3853-3857)
    const uint32_t f = cfg->savedetflag;
    const uint32_t partial = (cfg->medianum - 1) * (((f >> 1) & 1) + ((f >> 2) & 1) + ((f >> 3) & 1));
    cfg->his.maxmedia = cfg->medianum - 1;
    cfg->his.detnum = cfg->detnum;
    cfg->his.srcnum = cfg->srcnum;
    cfg->his.colcount = partial + (f & 1) + 3 * (((f >> 4) & 1) + ((f >> 5) & 1)) + ((f >> 6) & 1);
    cfg->his.savedetflag = cfg->savedetflag;
}

}  // namespace

// mcx_replayinit (src/mcx_utils.c:3624-3690): keep the detected photons of detector `replaydet`
// (all when <= 0) whose time of flight lies in [tstart, tend], with their seeds, detected weight
// exp(-sum mua_m ppath_m), time of flight sum ppath_m n_m / c0 and detector id.  detps holds
// dimdetps[1] records of dimdetps[0] floats (savedetflag with D and P); seeds arrive in
// cfg->replay.seed, seedbyte bytes per photon, and are compacted in place.  Sets nphoton.
extern "C" int mcxg_replayinit(Config* cfg, const float* detps, const int dimdetps[2], int seedbyte) {
    mcxg_clear_error();
    try {
        if (cfg->seed != kSEED_FROM_FILE) return 0;
        if (!detps) MCXG_RAISE(-6, "a replay needs the detected photons of the baseline run (detphotons)");
        if ((uint64_t)cfg->nphoton != (uint64_t)dimdetps[1]) MCXG_RAISE(-6, "the column numbers of detphotons and seed do not match");
        if (seedbyte == 0 || !cfg->replay.seed) MCXG_RAISE(-6, "the seed input is empty");
        const unsigned f = cfg->savedetflag;
        const int hasdetid = (int)(f & 0x1u);
        const int offset = (int)((f >> 1) & 1u) * ((int)cfg->medianum - 1);
        if ((!hasdetid && cfg->detnum > 1) || !((f >> 2) & 1u))
            MCXG_RAISE(-6, "please rerun the baseline simulation and save detector ID (D) and partial-path (P) using cfg.savedetflag='dp'");
        const int n = dimdetps[1], rec = dimdetps[0];
        free(cfg->replay.weight);
        free(cfg->replay.tof);
        free(cfg->replay.detid);
        cfg->replay.weight = (float*)malloc(std::max(1, n) * sizeof(float));
        cfg->replay.tof = (float*)calloc(std::max(1, n), sizeof(float));
        cfg->replay.detid = (int*)calloc(std::max(1, n), sizeof(int));
        int kept = 0;
        char* seeds = (char*)cfg->replay.seed;
        for (int i = 0; i < n; i++) {
            const float* r = detps + (size_t)i * rec;
            const int id = hasdetid ? (int)r[0] : 1;
            if (cfg->replaydet > 0 && cfg->replaydet != (id & 0xFFFF)) continue;
            float w = 1.f, tof = 0.f;
            for (int j = hasdetid; j < (int)cfg->medianum - 1 + hasdetid; j++) {
                float plen = r[offset + j];
                w *= expf(-cfg->prop[j - hasdetid + 1].mua * plen);
                plen *= cfg->unitinmm;
                tof += plen * kR_C0 * cfg->prop[j - hasdetid + 1].n;
            }
            if (tof < cfg->tstart || tof > cfg->tend) continue;
            if (i != kept) std::memmove(seeds + (size_t)kept * seedbyte, seeds + (size_t)i * seedbyte, seedbyte);
            cfg->replay.weight[kept] = w;
            cfg->replay.tof[kept] = tof;
            cfg->replay.detid[kept] = id;
            kept++;
        }
        cfg->nphoton = kept;
        return 0;
    } catch (const Error& e) {
        mcxg_set_error(e.id, e.msg.c_str());
        return e.id ? e.id : -1;
    }
}

extern "C" int mcxg_validatecfg(Config* cfg) {
    mcxg_clear_error();
    try {
        validate(cfg);
        return 0;
    } catch (const Error& e) {
        mcxg_set_error(e.id, e.msg.c_str());
        return e.id ? e.id : -1;
    }
}

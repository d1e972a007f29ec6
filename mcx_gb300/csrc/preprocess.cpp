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
// Out of this restatement (and rejected by the engine): seed files, polarised and
// split-voxel media, extra sources, shapes/JSON parsing.

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <algorithm>
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

void validate(Config* cfg) {
    // replay of saved photons (src/mcx_utils.c:1651-1664)
    if (cfg->seed == kSEED_FROM_FILE && (cfg->respin > 1 || cfg->respin < 0)) {
        cfg->respin = 1;
        if (cfg->flog) fprintf(cfg->flog, "WARNING: respin is disabled in the replay mode\n");
    }
    if (cfg->replaydet > (int)cfg->detnum) MCXG_RAISE(-4, "replay detector ID exceeds the maximum detector number");
    if (cfg->replaydet == -1 && cfg->detnum == 1) cfg->replaydet = 1;
    if (cfg->polprop || cfg->polmedianum) MCXG_RAISE(-6, "polarized media are not supported by the GB300 engine");
    if (cfg->extrasrclen) MCXG_RAISE(-6, "multiple sources are not supported by the GB300 engine");

    // mcx_validatecfg: grid-origin shift, time gates (src/mcx_utils.c:3761-3795)
    if (!cfg->issrcfrom0) {
        cfg->srcpos.x -= 1.f; cfg->srcpos.y -= 1.f; cfg->srcpos.z -= 1.f;
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

    if (cfg->steps.x != 1.f && cfg->unitinmm == 1.f) cfg->unitinmm = cfg->steps.x;
    if (cfg->unitinmm != 1.f) {
        cfg->steps.x = cfg->steps.y = cfg->steps.z = cfg->unitinmm;
        for (uint32_t i = 1; i < cfg->medianum; i++) {
            cfg->prop[i].mus *= cfg->unitinmm;
            cfg->prop[i].mua *= cfg->unitinmm;
        }
    }
    if (cfg->isrowmajor) {
        // C-order input: transpose to MCX's x-fastest order
        const uint3 d = cfg->dim;
        std::vector<uint32_t> tmp((size_t)d.x * d.y * d.z);
        for (uint32_t x = 0; x < d.x; x++)
            for (uint32_t y = 0; y < d.y; y++)
                for (uint32_t z = 0; z < d.z; z++)
                    tmp[(size_t)z * d.y * d.x + (size_t)y * d.x + x] = cfg->vol[((size_t)x * d.y + y) * d.z + z];
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
    cfg->savedetflag &= ~0x80u;       // no Stokes vector without polarisation
    if (cfg->issavedet && cfg->savedetflag == 0) cfg->savedetflag = 0x5;
    // per-voxel media have no labels: no per-medium record columns (src/mcx_utils.c:1801-1806)
    // per-voxel formats carry no per-medium slots (src/mcx_utils.c:1801-1803, mediabyte >= 100); for
    // mediabyte 96, 98 and 99 MCX keeps the flags and indexes the slots by the voxel word, past the
    // end of the record, so the engine clears them for every non-label format
    if (cfg->mediabyte > 4 && cfg->savedetflag) cfg->savedetflag &= ~(0x2u | 0x4u | 0x8u | 0x80u);
    if (cfg->issaveref) MCXG_RAISE(-6, "diffuse-reflectance output (issaveref) is not supported by the GB300 engine");

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

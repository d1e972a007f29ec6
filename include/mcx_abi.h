/*
 * mcx_abi.h -- the data layouts that cross the drop-in boundary.
 *
 * The MCX front-ends (the `mcx` CLI, the `pmcx` Python module and `mcxlab`) hand the
 * engine a `Config*` and a `GPUInfo*` and call the two entry points declared at the end
 * of this file.  For the engine to be a drop-in replacement, every struct here has to
 * agree with the front-end's definition byte for byte (field order, types, alignment,
 * total size).  The field names follow MCX so that code reading both sides lines up.
 *
 * Reference layouts this header must match (MCX v2025.10):
 *   Medium     src/mcx_utils.h:83-88     History  src/mcx_utils.h:115-132
 *   Replay     src/mcx_utils.h:138-143   GPUInfo  src/mcx_utils.h:149-166
 *   ExtraSrc   src/mcx_utils.h:102-107   Config   src/mcx_utils.h:172-285
 *   POLMedium  src/mcx_utils.h:94-100    enums    src/mcx_utils.h:70-73
 * The CPU test tests/test_abi_layout.py compiles a probe against this header and checks
 * every offset and size against the reference header when that is available, and against
 * the ctypes mirror in mcx_gb300/abi.py always.
 *
 * float4 / float3 / uint3 are CUDA's vector types: float4 is 16-byte aligned, the
 * three-component types are 4-byte aligned.
 */
#ifndef MCX_GB300_ABI_H
#define MCX_GB300_ABI_H

#include <stdio.h>
#include <stddef.h>
#include <vector_types.h>

#ifdef __cplusplus
extern "C" {
#endif

/* String and table capacities baked into the layout. */
#define MCXG_SESSION_LEN  256
#define MCXG_PATH_LEN     1024
#define MCXG_MAX_DEVICE   256
#define MCXG_LANG_LEN     32

/* Optical properties of one medium label: absorption and scattering coefficients
 * (1/mm, or 1/grid once scaled by unitinmm), anisotropy g and refractive index n. */
typedef struct MCXMedium {
    float mua;
    float mus;
    float g;
    float n;
} Medium;

/* Sphere population of a polarised medium: absorption (1/mm), radius (um), number density
 * (1/um^3), sphere and background refractive indices. */
typedef struct MCXPolarizeMedium {
    float mua;
    float r;
    float rho;
    float nsph;
    float nmed;
} POLMedium;

/* An additional source (multi-source runs). */
typedef struct MCXExtraSource {
    float4 srcpos;
    float4 srcdir;
    float4 srcparam1;
    float4 srcparam2;
} ExtraSrc;

/* 256-byte header of a detected-photon (.mch) record set. */
typedef struct MCXHistoryHeader {
    char         magic[4];
    unsigned int version;
    unsigned int maxmedia;
    unsigned int detnum;
    unsigned int colcount;
    unsigned int totalphoton;
    unsigned int detected;
    unsigned int savedphoton;
    float        unitinmm;
    unsigned int seedbyte;
    float        normalizer;
    int          respin;
    unsigned int srcnum;
    unsigned int savedetflag;
    unsigned int totalsource;
    int          reserved[1];
} History;

/* Inputs of a replay run (seeds, weights, times of flight, detector ids). */
typedef struct PhotonReplay {
    int*   detid;
    void*  seed;
    float* weight;
    float* tof;
} Replay;

/* One CUDA device as the front-ends see it; filled by mcx_list_gpu. */
typedef struct MCXGPUInfo {
    char         name[MCXG_SESSION_LEN];
    int          id;
    int          devcount;
    int          major;
    int          minor;
    size_t       globalmem;
    size_t       constmem;
    size_t       sharedmem;
    int          regcount;
    int          clock;
    int          sm;
    int          core;
    int          autoblock;
    int          autothread;
    unsigned int maxgate;
    int          maxmpthread;
} GPUInfo;

/* The complete simulation description shared by every front-end.  Fields the engine
 * reads or writes are described in mcx_gb300/csrc/engine.cu; the rest are carried. */
typedef struct MCXConfig {
    size_t       nphoton;
    unsigned int nblocksize;
    unsigned int nthread;
    int          seed;

    float4       srcpos;          /* x,y,z in grid units, w = initial packet weight */
    float4       srcdir;          /* unit direction, w = focal length */
    float4       srciquv;
    float        tstart;
    float        tstep;
    float        tend;
    float3       steps;           /* voxel edge lengths in mm */

    uint3        dim;
    uint3        crop0;
    uint3        crop1;
    unsigned int medianum;        /* rows of prop, including label 0 */
    unsigned int polmedianum;
    unsigned int detnum;
    unsigned int maxdetphoton;
    float        detradius;
    float        sradius;

    Medium*      prop;
    POLMedium*   polprop;
    float4*      detpos;          /* x,y,z,radius per detector */
    float4*      smatrix;

    unsigned int maxgate;
    int          respin;
    int          printnum;
    int          gpuid;

    unsigned int* vol;            /* uint32 per voxel, x fastest; bit 31 = detector mask */
    char         session[MCXG_SESSION_LEN];
    char         isrowmajor;
    char         isreflect;
    char         isref3;
    char         isrefint;
    char         isnormalized;
    char         issavedet;
    char         issave2pt;
    char         isgpuinfo;
    char         isspecular;
    char         issrcfrom0;
    char         isdumpmask;
    char         autopilot;
    char         issaveseed;
    char         issaveexit;
    char         issaveref;
    char         ismomentum;
    char         istrajstokes;
    char         isdumpjson;
    char         internalsrc;
    int          zipid;
    char         srctype;
    char         outputtype;
    char         outputformat;
    char         faststep;
    float        minenergy;
    float        unitinmm;
    float        omega;
    float        lambda;
    FILE*        flog;
    History      his;
    float*       exportfield;     /* accumulated (+=) flux, caller-owned when non-NULL */
    float*       exportdetected;  /* detected-photon records, realloc'ed by the engine */
    unsigned long int detectedcount;
    char         rootpath[MCXG_PATH_LEN];
    char*        shapedata;
    char*        extrajson;
    int          maxvoidstep;
    int          voidtime;
    float4       srcparam1;
    float4       srcparam2;       /* after preprocessing: .z/.w hold launch voxel/medium bits */
    unsigned int srcnum;
    float*       srcpattern;
    Replay       replay;
    void*        seeddata;
    int          replaydet;
    char         seedfile[MCXG_PATH_LEN];
    char         jsonfile[MCXG_PATH_LEN];
    unsigned int debuglevel;
    unsigned int savedetflag;
    char         deviceid[MCXG_MAX_DEVICE];
    float        workload[MCXG_MAX_DEVICE];
    int          parentid;
    unsigned int runtime;         /* kernel milliseconds, written by the engine */
    char         langid[MCXG_LANG_LEN];

    double       energytot;
    double       energyabs;
    double       energyesc;
    float        normalizer;
    unsigned int maxjumpdebug;
    unsigned int debugdatalen;
    unsigned int gscatter;
    float*       exportdebugdata;
    unsigned int mediabyte;
    float*       dx;
    float*       dy;
    float*       dz;
    char         bc[13];          /* faces -x,-y,-z,+x,+y,+z then detector flags, NUL */
    unsigned int nphase;
    float*       invcdf;
    unsigned int nangle;
    float*       angleinvcdf;
    int          srcid;
    unsigned int extrasrclen;
    ExtraSrc*    srcdata;
} Config;

/* Enumerations whose numeric values are part of the Config contract
 * (src/mcx_utils.h:70-73). */
enum { otFlux, otFluence, otEnergy, otJacobian, otWP, otDCS, otRF, otL, otRFmus, otWLTOF, otWPTOF };
enum { mpStandalone, mpMATLAB, mpPython };
enum { bcUnknown, bcReflect, bcAbsorb, bcMirror, bcCyclic };

/*
 * The drop-in entry points (reference declarations: src/mcx_core.h:200-201).
 *
 * mcx_list_gpu: enumerates CUDA devices into a calloc'ed GPUInfo array (the caller frees it),
 * compacts cfg->deviceid from a '0'/'1' mask into a 1-based id list and returns the number of
 * active devices (reference behaviour: src/mcx_core.cu:2621-2726).
 *
 * mcx_run_simulation: runs the photon-transport simulation described by an already
 * preprocessed Config on the device selected by the calling OpenMP thread, accumulates the
 * fluence into cfg->exportfield, appends detected photons to cfg->exportdetected and writes
 * runtime, energies and the normaliser back into cfg (reference: src/mcx_core.cu:2740-4110).
 * Errors are reported through mcx_error() when a front-end provides it; otherwise they are
 * recorded and readable with mcxg_last_error() (include/mcx_gb300.h).
 */
void mcx_run_simulation(Config* cfg, GPUInfo* gpu);
int  mcx_list_gpu(Config* cfg, GPUInfo** info);

#ifdef __cplusplus
}
#endif

#endif /* MCX_GB300_ABI_H */

// mcxg_common.h -- constants and small helpers shared by the engine's host and device code.
#pragma once

#include <cstdint>
#include <cfloat>
#include <string>

namespace mcxg {

// Values that are part of MCX's data contract (src/mcx_const.h:51-60, src/mcx_utils.h:48).
constexpr float    kEPS       = FLT_EPSILON;              // round-off guard used throughout MCX
constexpr uint32_t kDET_MASK  = 0x80000000u;              // bit 31 of a uint32 voxel: detector voxel
constexpr uint32_t kMED_MASK  = 0x7FFFFFFFu;              // remaining bits: medium label
constexpr uint32_t kOUT_MIN   = 0xFFFFFFFFu;              // photon left through a x/y/z = 0 face
constexpr uint32_t kOUT_MAX   = 0x7FFFFFFFu;              // photon left through a far face
constexpr float    kR_C0      = 3.335640951981520e-12f;   // 1/c in s/mm
constexpr float    kTWO_PI    = 6.28318530717959f;
constexpr float    kPI        = 3.1415926535897932f;
constexpr float    kR_PI      = 0.318309886183791f;         // 1/pi
constexpr int      kSEED_FROM_FILE = -999;
constexpr int      kFILL_MAXDETPHOTON = 3;
constexpr size_t   kSeedBytes = 16;                      // saved generator state per photon: RAND_BUF_LEN x 8 B

// Engine limits.  The GB300 engine keeps one byte per voxel: bit 7 is the detector mask and
// bits 0-6 the medium label, so a run may use at most 128 property rows (labels 0..127).
constexpr int      kMaxMedia     = 128;
constexpr uint8_t  kLabelDet     = 0x80;
constexpr uint8_t  kLabelMask    = 0x7F;
constexpr int      kMaxDetectors = 256;

// Boundary-condition codes stored in Config::bc (src/mcx_utils.h:73).
enum : int { BC_UNKNOWN = 0, BC_REFLECT = 1, BC_ABSORB = 2, BC_MIRROR = 3, BC_CYCLIC = 4 };

// An engine error: raised inside the engine, turned into mcx_error() (or the recorded last
// error) at the C-ABI boundary.
struct Error {
    int id;
    std::string msg;
    const char* file;
    int line;
};

[[noreturn]] void raise(int id, const std::string& msg, const char* file, int line);
#define MCXG_RAISE(id, msg) ::mcxg::raise((id), (msg), __FILE__, __LINE__)

}  // namespace mcxg

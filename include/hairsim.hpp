// hairsim.hpp -- C++17 wrapper of the C-ABI in hairsim.h, shaped like the
// reference's Hair class (src/fx/hair.h:24-121) so that its call sites keep
// their form: init(), setup(roots, normals), set_bounding_sphere(s),
// update(dt), initialized(), deinit(), plus readback of the control points.
//
// Header only; link against libhairsim.so. Errors throw hs::Error with the
// library's status and message.
#ifndef HAIRSIM_HPP_
#define HAIRSIM_HPP_

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "hairsim.h"

namespace hs {

class Error : public std::runtime_error {
 public:
  Error(hs_status st, const std::string& where)
      : std::runtime_error(where + ": " + hs_last_error_string()), status(st) {}
  hs_status status;
};

inline void check(hs_status st, const char* where) {
  if (st != HS_OK) throw Error(st, where);
}

// The reference's UI parameters that reach the simulation
// (Parameters_t, src/fx/hair.h:27-51).
struct HairParameters {
  float max_length = 0.50f;    // sim.maxlength
  float length_scale = 1.45f;  // render.lengthScale, passed as uScaleFactor
  uint64_t seed = 0;           // stands in for the time-seeded rand()
};

class Hair {
 public:
  Hair() = default;
  explicit Hair(HairParameters p) : params_(p) {}
  Hair(const Hair&) = delete;
  Hair& operator=(const Hair&) = delete;
  ~Hair() { deinit(); }

  // Hair::init (src/fx/hair.cc:26-40): the simulation needs a context.
  void init() {
    if (!ctx_) check(hs_create(&ctx_), "hs_create");
  }

  // Hair::deinit (src/fx/hair.cc:66-87).
  void deinit() noexcept {
    if (groom_) hs_groom_destroy(groom_);
    groom_ = nullptr;
    if (ctx_) hs_destroy(ctx_);
    ctx_ = nullptr;
    nroots_ = 0;
  }

  // Hair::setup (src/fx/hair.cc:42-64): one strand per scalp vertex; roots
  // and normals are the mesh's positions and normals (3 floats each).
  void setup(const std::vector<float>& roots, const std::vector<float>& normals) {
    if (!ctx_) throw Error(HS_ERR_NOT_INITIALIZED, "Hair::setup before init");
    if (roots.size() != normals.size() || roots.size() % 3 != 0)
      throw Error(HS_ERR_INVALID_ARG, "Hair::setup: roots and normals must be 3 floats per vertex");
    hs_strand_params sp;
    hs_strand_params_reference(&sp);
    sp.max_length = params_.max_length;
    sp.seed = params_.seed;
    hs_sim_params sim;
    hs_sim_params_reference(&sim);
    sim.length_scale = params_.length_scale;
    if (groom_) hs_groom_destroy(groom_);
    groom_ = nullptr;
    const uint32_t n = static_cast<uint32_t>(roots.size() / 3);
    check(hs_groom_init(ctx_, roots.data(), normals.data(), n, &sp, &sim, &groom_), "hs_groom_init");
    nroots_ = n;
  }

  // Hair::set_bounding_sphere (src/fx/hair.h:72-74).
  void set_bounding_sphere(const std::array<float, 4>& xyzr) noexcept { bsphere_ = xyzr; }

  // Hair::update (src/fx/hair.cc:89-125): silently does nothing before
  // setup, as the reference does (:90-93).
  void update(float dt) {
    if (!initialized()) return;
    check(hs_set_bounding_sphere(groom_, bsphere_.data()), "hs_set_bounding_sphere");
    check(hs_update(groom_, dt), "hs_update");
  }

  // Hair::initialized (src/fx/hair.h:76-78).
  bool initialized() const noexcept { return nroots_ != 0; }
  int nroots() const noexcept { return static_cast<int>(nroots_); }

  // The control points the renderer consumes: (x, y, z, restlength) per
  // point, strand-major (src/fx/hair.cc:369-392).
  std::vector<float> readback() const {
    std::vector<float> out(static_cast<size_t>(nroots_) * 4 * points(), 0.0f);
    if (initialized()) check(hs_readback(groom_, out.data(), out.size()), "hs_readback");
    return out;
  }

  uint32_t points() const {
    uint32_t ns = 0, np = 0;
    if (groom_) hs_groom_info(groom_, &ns, &np);
    return np;
  }
  hs_groom* groom() const noexcept { return groom_; }
  hs_ctx* context() const noexcept { return ctx_; }

 private:
  HairParameters params_;
  hs_ctx* ctx_ = nullptr;
  hs_groom* groom_ = nullptr;
  uint32_t nroots_ = 0;
  std::array<float, 4> bsphere_{0.0f, 0.0f, 0.0f, 1.0f};  // uBoundingSphere default (cs_simulation.glsl:43)
};

}  // namespace hs

#endif  // HAIRSIM_HPP_

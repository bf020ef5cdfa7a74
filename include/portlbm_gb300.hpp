// portlbm_gb300.hpp — C++ drop-in for PortLBM's public API on top of the C ABI in plbm_c.h.
//
// Mirrors (SC-SGS/PortLBM, paths relative to that project):
//   lbm::core::Properties                       include/lbm/core/properties.hpp:30-166
//   lbm::execution::AlgorithmHandler            include/lbm/execution/algorithm_handler.hpp:40-156
//   lbm::create_handler(Properties / path)      include/lbm/portlbm_factory.hpp:59,73
//   lbm::exceptions::{Exception, json::PropertyArgumentException, algorithm::WaitException}
//                                               include/lbm/exceptions/exceptions.hpp:31-150
// A reference user replaces `#include <lbm/portlbm.hpp>` with this header and links libplbm.so;
// the calls, argument meanings (inner extents in, stored extents out) and exceptions are the same.
// Header-only; no CUDA headers needed by the includer.
#ifndef PORTLBM_GB300_HPP
#define PORTLBM_GB300_HPP

#include "plbm_c.h"

#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace lbm {

#ifdef USE_FLOAT
using real_type = float;
#else
using real_type = double;
#endif

namespace exceptions {
class Exception : public std::runtime_error {
  public:
    explicit Exception(const std::string &m) : std::runtime_error(m) {}
};
namespace json {
class PropertyArgumentException : public Exception {
  public:
    using Exception::Exception;
};
}  // namespace json
namespace algorithm {
class WaitException : public Exception {
  public:
    using Exception::Exception;
};
}  // namespace algorithm
class CudaException : public Exception {
  public:
    using Exception::Exception;
};
}  // namespace exceptions

namespace detail {
inline void check(int rc, const plbm_handler *h)
{
    if (rc == PLBM_OK) return;
    const std::string msg = plbm_last_error(h);
    switch (rc) {
    case PLBM_ERR_PROPERTY: throw exceptions::json::PropertyArgumentException(msg);
    case PLBM_ERR_WAIT: throw exceptions::algorithm::WaitException(msg);
    case PLBM_ERR_CUDA:
    case PLBM_ERR_NO_DEVICE: throw exceptions::CudaException(msg);
    default: throw exceptions::Exception(msg);
    }
}
}  // namespace detail

namespace core {

// Properties as the reference constructs it: inner extents in, two ghost layers added.
struct Properties {
    std::string algorithm, data_layout;
    bool debug_mode;
    unsigned int work_group_size, time_steps, frame_update_interval;
    std::string scenario;
    unsigned int vertical_nodes, horizontal_nodes, total_unexpanded_node_count, domain_node_count;
    real_type inlet_velocity_x, inlet_velocity_y, inlet_density;
    real_type outlet_velocity_x, outlet_velocity_y, outlet_density;
    real_type relaxation_time;
    std::string settings_path;

    Properties(std::string algorithm_, std::string data_layout_, bool debug_mode_, unsigned int work_group_size_,
               unsigned int time_steps_, unsigned int frame_update_interval_, std::string scenario_,
               unsigned int vertical_nodes_, unsigned int horizontal_nodes_, real_type ivx, real_type ivy,
               real_type irho, real_type ovx, real_type ovy, real_type orho, real_type tau)
        : algorithm(std::move(algorithm_)), data_layout(std::move(data_layout_)), debug_mode(debug_mode_),
          work_group_size(work_group_size_), time_steps(time_steps_), frame_update_interval(frame_update_interval_),
          scenario(std::move(scenario_)), vertical_nodes(vertical_nodes_ + 2), horizontal_nodes(horizontal_nodes_ + 2),
          total_unexpanded_node_count((vertical_nodes_ + 2) * (horizontal_nodes_ + 2)),
          domain_node_count(vertical_nodes_ * horizontal_nodes_), inlet_velocity_x(ivx), inlet_velocity_y(ivy),
          inlet_density(irho), outlet_velocity_x(ovx), outlet_velocity_y(ovy), outlet_density(orho),
          relaxation_time(tau)
    {
    }

    plbm_properties to_c() const
    {
        plbm_properties c{};
        c.algorithm = algorithm.c_str();
        c.data_layout = data_layout.c_str();
        c.debug_mode = debug_mode;
        c.work_group_size = work_group_size;
        c.time_steps = time_steps;
        c.frame_update_interval = frame_update_interval;
        c.scenario = scenario.c_str();
        c.vertical_nodes = vertical_nodes - 2;
        c.horizontal_nodes = horizontal_nodes - 2;
        c.inlet_velocity_x = inlet_velocity_x;
        c.inlet_velocity_y = inlet_velocity_y;
        c.inlet_density = inlet_density;
        c.outlet_velocity_x = outlet_velocity_x;
        c.outlet_velocity_y = outlet_velocity_y;
        c.outlet_density = outlet_density;
        c.relaxation_time = relaxation_time;
        return c;
    }

    // Properties::validate (src/lbm/core/simulation.cpp:60-125).
    void validate() const
    {
        const plbm_properties c = to_c();
        detail::check(plbm_validate(&c), nullptr);
    }
};

}  // namespace core

namespace execution {

class AlgorithmHandler {
  public:
    size_t processing_element_constraint = 1024;

    explicit AlgorithmHandler(plbm_handler *h) : h_(h) { sync(); }
    ~AlgorithmHandler() { plbm_destroy(h_); }
    AlgorithmHandler(const AlgorithmHandler &) = delete;
    AlgorithmHandler &operator=(const AlgorithmHandler &) = delete;

    void initialize() { detail::check(plbm_initialize(h_), h_); }
    void start() { detail::check(plbm_start(h_), h_); }
    void pause() { detail::check(plbm_pause(h_), h_); }
    bool is_finished() const
    {
        int f = 0;
        plbm_is_finished(h_, &f);
        return f != 0;
    }
    void block_until_finished()
    {
        detail::check(plbm_block_until_finished(h_), h_);
        sync();
    }

    // The reference returns references to host vectors that the worker thread refreshes on frame
    // steps; these vectors are refreshed from the library's host arrays when a call returns.
    std::vector<real_type> &get_densities() const { return pull(PLBM_DENSITY); }
    std::vector<real_type> &get_x_velocities() const { return pull(PLBM_X_VELOCITY); }
    std::vector<real_type> &get_y_velocities() const { return pull(PLBM_Y_VELOCITY); }
    std::vector<real_type> &get_absolute_velocities() const { return pull(PLBM_ABS_VELOCITY); }

    unsigned int get_horizontal_nodes() const
    {
        unsigned hn = 0, vn = 0;
        plbm_get_extents(h_, &hn, &vn);
        return hn;
    }
    unsigned int get_vertical_nodes() const
    {
        unsigned hn = 0, vn = 0;
        plbm_get_extents(h_, &hn, &vn);
        return vn;
    }
    real_type get_inlet_density() const { return props().inlet_density; }
    real_type get_outlet_density() const { return props().outlet_density; }
    real_type get_progress() const
    {
        double p = 0;
        plbm_get_progress(h_, &p);
        return (real_type)p;
    }
    real_type get_last_frametime() const
    {
        double ms = 0;
        plbm_get_last_frametime(h_, &ms);
        return (real_type)ms;
    }
    unsigned int get_current_iteration() const
    {
        unsigned it = 0;
        plbm_get_current_iteration(h_, &it);
        return it;
    }
    plbm_properties props() const
    {
        plbm_properties c{};
        plbm_get_properties(h_, &c);
        return c;
    }
    plbm_handler *native() const { return h_; }

  private:
    plbm_handler *h_;
    mutable std::vector<real_type> res_[4];

    std::vector<real_type> &pull(int which) const
    {
        const double *d = nullptr;
        size_t n = 0;
        plbm_get_results(h_, which, &d, &n);
        res_[which].assign(d, d + n);
        return res_[which];
    }
    void sync() const
    {
        for (int i = 0; i < 4; ++i) pull(i);
    }
};

}  // namespace execution

// lbm::create_handler (portlbm_factory.hpp:59,73); `options` selects the arithmetic form, etc.
inline std::unique_ptr<execution::AlgorithmHandler> create_handler(const core::Properties &props,
                                                                   const plbm_options *options = nullptr)
{
    const plbm_properties c = props.to_c();
    plbm_handler *h = nullptr;
    detail::check(plbm_create(&c, options, &h), nullptr);
    return std::make_unique<execution::AlgorithmHandler>(h);
}

inline std::unique_ptr<execution::AlgorithmHandler> create_handler(const std::string &settings_path,
                                                                   const plbm_options *options = nullptr)
{
    plbm_handler *h = nullptr;
    detail::check(plbm_create_from_json(settings_path.c_str(), options, &h), nullptr);
    return std::make_unique<execution::AlgorithmHandler>(h);
}

}  // namespace lbm

#endif  // PORTLBM_GB300_HPP

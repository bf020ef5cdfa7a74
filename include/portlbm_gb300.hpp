// portlbm_gb300.hpp — C++ drop-in for PortLBM's public API on top of the C ABI in plbm_c.h.
//
// Mirrors (SC-SGS/PortLBM, paths relative to that project):
//   lbm::core::Properties                       include/lbm/core/properties.hpp:30-166
//   lbm::core::Domain                           include/lbm/core/domain.hpp:29-85
//   lbm::execution::AlgorithmHandler (abstract) include/lbm/execution/algorithm_handler.hpp:40-156
//   lbm::execution::CUDAAlgorithmHandler        the concrete handler, in the place of
//                                               include/lbm/execution/sycl_algorithm_handler.hpp:45-455
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

    // The inverse of to_c(): the C struct carries inner extents, as the constructor takes them.
    static Properties from_c(const plbm_properties &c)
    {
        return Properties(c.algorithm ? c.algorithm : "", c.data_layout ? c.data_layout : "", c.debug_mode != 0,
                          c.work_group_size, c.time_steps, c.frame_update_interval, c.scenario ? c.scenario : "",
                          c.vertical_nodes, c.horizontal_nodes, (real_type)c.inlet_velocity_x,
                          (real_type)c.inlet_velocity_y, (real_type)c.inlet_density, (real_type)c.outlet_velocity_x,
                          (real_type)c.outlet_velocity_y, (real_type)c.outlet_density, (real_type)c.relaxation_time);
    }

    // Properties::validate (src/lbm/core/simulation.cpp:60-125).
    void validate() const
    {
        const plbm_properties c = to_c();
        detail::check(plbm_validate(&c), nullptr);
    }
};

// core::Domain (include/lbm/core/domain.hpp:29-85): the padded / buffered extents and the
// subdomain (work-group tile) decomposition of one algorithm, computed as
// src/lbm/core/simulation.cpp:194-382 does.
class Domain {
  public:
    unsigned int total_node_count = 0;
    unsigned int horizontal_nodes = 0;
    unsigned int vertical_nodes = 0;
    unsigned int subdomain_vertical_nodes = 0;
    unsigned int subdomain_horizontal_nodes = 0;
    unsigned int subdomain_count_vertical = 0;
    unsigned int subdomain_count_horizontal = 0;

    Domain() = default;
    // Domain(Properties&): throws PropertyArgumentException where the reference's swap set-up
    // rejects the work-group size (below 6).  The library does that settings.json rewrite when a
    // handler is created from the file; this constructor leaves the file alone.
    explicit Domain(Properties &properties)
    {
        const plbm_properties c = properties.to_c();
        unsigned v[7] = { 0, 0, 0, 0, 0, 0, 0 };
        detail::check(plbm_compute_domain(&c, v), nullptr);
        *this = Domain(v);
    }
    // From the seven values plbm_compute_domain / plbm_get_domain write, in the field order above.
    explicit Domain(const unsigned (&v)[7])
        : total_node_count(v[0]), horizontal_nodes(v[1]), vertical_nodes(v[2]), subdomain_vertical_nodes(v[3]),
          subdomain_horizontal_nodes(v[4]), subdomain_count_vertical(v[5]), subdomain_count_horizontal(v[6])
    {
    }
};

}  // namespace core

namespace execution {

// The abstract handler interface (algorithm_handler.hpp:40-156): callers hold a
// std::unique_ptr<AlgorithmHandler> from lbm::create_handler and use only these members.
class AlgorithmHandler {
  public:
    // Upper bound on the processing elements (threads) per work-group; the concrete handler sets
    // the device's maximum, as the reference does (sycl_algorithm_handler.hpp:302).
    size_t processing_element_constraint;

    virtual ~AlgorithmHandler() = default;

    virtual void initialize() = 0;
    virtual void start() = 0;
    virtual void pause() = 0;
    virtual bool is_finished() const = 0;
    virtual void block_until_finished() = 0;

    virtual std::vector<real_type> &get_densities() const = 0;
    virtual std::vector<real_type> &get_x_velocities() const = 0;
    virtual std::vector<real_type> &get_y_velocities() const = 0;
    virtual std::vector<real_type> &get_absolute_velocities() const = 0;

    // stored extents of the unexpanded domain (inner + 2 ghost layers)
    virtual unsigned int get_horizontal_nodes() const = 0;
    virtual unsigned int get_vertical_nodes() const = 0;
    virtual real_type get_inlet_density() const = 0;
    virtual real_type get_outlet_density() const = 0;
    virtual real_type get_progress() const = 0;
    virtual real_type get_last_frametime() const = 0;
    virtual unsigned int get_current_iteration() const = 0;

    virtual const core::Properties &get_properties() const = 0;
    virtual const core::Domain &get_domain() const = 0;

  protected:
    explicit AlgorithmHandler(size_t constraint) : processing_element_constraint(constraint) {}
};

// The CUDA implementation behind lbm::create_handler (the counterpart of SYCLAlgorithmHandler,
// sycl_algorithm_handler.hpp:45-455): owns one libplbm handle.
class CUDAAlgorithmHandler final : public AlgorithmHandler {
  public:
    // every CUDA device's maxThreadsPerBlock
    static constexpr size_t max_work_group_size = 1024;

    explicit CUDAAlgorithmHandler(plbm_handler *h, std::string settings_path = std::string())
        : AlgorithmHandler(max_work_group_size), h_(h), settings_path_(std::move(settings_path))
    {
        refresh_description();
        sync();
    }
    ~CUDAAlgorithmHandler() override { plbm_destroy(h_); }
    CUDAAlgorithmHandler(const CUDAAlgorithmHandler &) = delete;
    CUDAAlgorithmHandler &operator=(const CUDAAlgorithmHandler &) = delete;

    // Rebuilds the simulation; a handler made from settings.json re-reads it, so the properties
    // and the domain are taken afresh.
    void initialize() override
    {
        detail::check(plbm_initialize(h_), h_);
        refresh_description();
        sync();
    }
    void start() override { detail::check(plbm_start(h_), h_); }
    void pause() override { detail::check(plbm_pause(h_), h_); }
    bool is_finished() const override
    {
        int f = 0;
        plbm_is_finished(h_, &f);
        return f != 0;
    }
    void block_until_finished() override
    {
        detail::check(plbm_block_until_finished(h_), h_);
        sync();
    }

    // The reference returns references to host vectors that the worker thread refreshes on frame
    // steps; these vectors are refreshed from the library's host arrays when a call returns.
    std::vector<real_type> &get_densities() const override { return pull(PLBM_DENSITY); }
    std::vector<real_type> &get_x_velocities() const override { return pull(PLBM_X_VELOCITY); }
    std::vector<real_type> &get_y_velocities() const override { return pull(PLBM_Y_VELOCITY); }
    std::vector<real_type> &get_absolute_velocities() const override { return pull(PLBM_ABS_VELOCITY); }

    unsigned int get_horizontal_nodes() const override
    {
        unsigned hn = 0, vn = 0;
        plbm_get_extents(h_, &hn, &vn);
        return hn;
    }
    unsigned int get_vertical_nodes() const override
    {
        unsigned hn = 0, vn = 0;
        plbm_get_extents(h_, &hn, &vn);
        return vn;
    }
    real_type get_inlet_density() const override { return props_->inlet_density; }
    real_type get_outlet_density() const override { return props_->outlet_density; }
    real_type get_progress() const override
    {
        double p = 0;
        plbm_get_progress(h_, &p);
        return (real_type)p;
    }
    real_type get_last_frametime() const override
    {
        double ms = 0;
        plbm_get_last_frametime(h_, &ms);
        return (real_type)ms;
    }
    unsigned int get_current_iteration() const override
    {
        unsigned it = 0;
        plbm_get_current_iteration(h_, &it);
        return it;
    }
    const core::Properties &get_properties() const override { return *props_; }
    const core::Domain &get_domain() const override { return dom_; }

    // The C ABI handle, for the measurement and batch entry points of plbm_c.h.
    plbm_handler *native() const { return h_; }

  private:
    plbm_handler *h_;
    std::string settings_path_;
    std::unique_ptr<core::Properties> props_;
    core::Domain dom_;
    mutable std::vector<real_type> res_[4];

    void refresh_description()
    {
        plbm_properties c{};
        plbm_get_properties(h_, &c);
        props_ = std::make_unique<core::Properties>(core::Properties::from_c(c));
        props_->settings_path = settings_path_;
        unsigned v[7] = { 0, 0, 0, 0, 0, 0, 0 };
        plbm_get_domain(h_, v);
        dom_ = core::Domain(v);
    }
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
    return std::make_unique<execution::CUDAAlgorithmHandler>(h, props.settings_path);
}

inline std::unique_ptr<execution::AlgorithmHandler> create_handler(const std::string &settings_path,
                                                                   const plbm_options *options = nullptr)
{
    plbm_handler *h = nullptr;
    detail::check(plbm_create_from_json(settings_path.c_str(), options, &h), nullptr);
    return std::make_unique<execution::CUDAAlgorithmHandler>(h, settings_path);
}

}  // namespace lbm

#endif  // PORTLBM_GB300_HPP

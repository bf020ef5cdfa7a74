// Placeholder for nlohmann/json — TEST INFRASTRUCTURE.  The oracle build does not compile the
// reference's settings I/O; ref_driver.cpp provides json_to_properties/properties_to_json stubs.
#pragma once
namespace nlohmann { struct json {}; }

/* Empty base class the reference's tree_topology derives from.  Oracle build only. */
#pragma once
namespace flecsi {
namespace data {
class data_client_t {};
} // namespace data
} // namespace flecsi

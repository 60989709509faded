// Oracle test infrastructure: empty stand-in for boost::serialization::access,
// which the SOUFFLE sources only name as a friend class.
#ifndef ORACLE_SHIM_BOOST_SERIALIZATION_ACCESS_HPP
#define ORACLE_SHIM_BOOST_SERIALIZATION_ACCESS_HPP
namespace boost {
namespace serialization {
class access {};
}  // namespace serialization
}  // namespace boost
#endif

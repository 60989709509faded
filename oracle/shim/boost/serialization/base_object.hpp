#include <boost/serialization/access.hpp>

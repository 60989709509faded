#include <boost/serialization/access.hpp>
#include <vector>

/* Build shim for compiling the CIFlow reference sources as a test oracle.
 * The reference only uses the namespace alias when its 64-bit bitstring
 * type is selected, so an empty namespace is enough. */
#pragma once
namespace boost { namespace multiprecision {} }

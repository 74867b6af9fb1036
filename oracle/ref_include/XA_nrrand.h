/* Declaration of the Gaussian deviate that TemsimLibrary/autoslic.cpp:137
 * includes from the (absent) XArrayLibrary.  Defined in oracle/ref_driver.cpp.
 * TEST INFRASTRUCTURE ONLY. */
#pragma once
double gasdev(long *idum);

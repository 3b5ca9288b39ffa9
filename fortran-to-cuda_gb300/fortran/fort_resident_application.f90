! The one residency domain of an application that keeps none of its own: the
! object the generated directives and call blocks name (`resident`).
module fort_resident_application
  use fort_resident_domain, only: resident_domain, resident_require
  implicit none
  private
  public :: resident, resident_require
  type(resident_domain), save, target :: resident
end module fort_resident_application
